// Kernels of the batch engine (batch.hpp): one persistent launch per fused
// layer over the tiles of many registers, the |0...0> initialisation of a
// wave of registers, and batched Pauli-sum reductions.
#include "batch.hpp"

#include <type_traits>
#include "tile_reg.cuh"

namespace plgb {

template <class T, bool OCC>
__global__ void __launch_bounds__(256, OCC ? 2 : 1)
    k_tile_reg_batch(const BatchTileItem<T> *__restrict__ items, int nitems, u64 total_tiles) {
    extern __shared__ unsigned char smraw[];
    cx<T> *tile = reinterpret_cast<cx<T> *>(smraw);
    __shared__ TileShared<T> sh;
    __shared__ TilePassDesc sd;
    const RegOpS<T> *recs = nullptr; // staged op records of the current item
    int cur = -1;
    for (u64 gt = blockIdx.x; gt < total_tiles; gt += gridDim.x) {
        // item owning global tile gt: the last one whose tile_begin <= gt
        int lo = 0, hi = nitems - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (items[mid].tile_begin <= gt) {
                lo = mid;
            } else {
                hi = mid - 1;
            }
        }
        if (lo != cur) { // block-uniform: every thread found the same item
            __syncthreads();
            if (threadIdx.x == 0) {
                sd = items[lo].desc;
            }
            recs = op_records<T, true>(smraw + (sizeof(cx<T>) << items[lo].desc.t), items[lo].ops, items[lo].desc);
            __syncthreads();
            cur = lo;
        }
        const BatchTileItem<T> &it = items[lo];
        tile_reg_run<T>(it.sv, it.sv, sd, it.ops, it.forms, it.tables, it.stages, gt - it.tile_begin, tile, sh, recs);
    }
}

template <class T, bool OCC>
static void launch_batch_impl(cudaStream_t s, int t, const BatchTileItem<T> *items, int nitems, u64 total_tiles,
                              int max_ops) {
    const int threads = 1 << (t - kRegBits);
    const size_t smem = (sizeof(cx<T>) << t) + op_record_bytes<T, true>(max_ops);
    static bool attr = false;
    if (!attr) {
        cuda_check(cudaFuncSetAttribute(k_tile_reg_batch<T, OCC>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        200 * 1024), "tile_reg_batch smem attribute");
        attr = true;
    }
    int per_sm = 1;
    cuda_check(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_tile_reg_batch<T, OCC>, threads, smem),
               "occupancy");
    if (per_sm < 1) {
        throw std::runtime_error("batched tile pass: tile does not fit one SM");
    }
    const u64 cap = static_cast<u64>(LaunchGeom::sm_count()) * static_cast<u64>(per_sm);
    const unsigned grid = static_cast<unsigned>(total_tiles < cap ? total_tiles : cap);
    k_tile_reg_batch<T, OCC><<<grid, threads, smem, s>>>(items, nitems, total_tiles);
    cuda_check(cudaGetLastError(), "k_tile_reg_batch launch");
    note_launch();
}

template <class T>
void launch_tile_reg_batch(cudaStream_t s, int t, const BatchTileItem<T> *items, int nitems, u64 total_tiles,
                           int max_ops) {
    if (t < kMinRegTileBits || t > 12 || nitems < 1 || total_tiles < 1 || max_ops > kMaxOpsPerPass) {
        throw std::runtime_error("batched tile pass: unsupported geometry");
    }
    if (tile_variant_occ(std::is_same_v<T, float> ? 64 : 128)) {
        launch_batch_impl<T, true>(s, t, items, nitems, total_tiles, max_ops);
    } else {
        launch_batch_impl<T, false>(s, t, items, nitems, total_tiles, max_ops);
    }
}

// Entry j of a table: the product of its factors' values at the bits of j.
__global__ void k_expand_tables(const DevRecipe *__restrict__ rec, int nrec, u64 total, int enc) {
    for (u64 e = static_cast<u64>(blockIdx.x) * blockDim.x + threadIdx.x; e < total;
         e += static_cast<u64>(gridDim.x) * blockDim.x) {
        int lo = 0, hi = nrec - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (rec[mid].entry_begin <= e) {
                lo = mid;
            } else {
                hi = mid - 1;
            }
        }
        const DevRecipe &r = rec[lo];
        const u32 j = static_cast<u32>(e - r.entry_begin);
        cx<double> v{1.0, 0.0};
        for (int f = 0; f < r.nfac; f++) {
            const TableFactor &tf = r.fac[f];
            unsigned k = 0;
            for (int b = 0; b < tf.nb; b++) {
                k = (k << 1) | ((j >> tf.pos[b]) & 1u);
            }
            v = v * tf.val[k];
        }
        if (enc == 0) {
            static_cast<cx<float> *>(r.dst)[j] = cx<float>{static_cast<float>(v.x), static_cast<float>(v.y)};
        } else if (enc == 1) {
            static_cast<cx<double> *>(r.dst)[j] = v;
        } else {
            static_cast<cx<df> *>(r.dst)[j] = cx<df>{df(v.x), df(v.y)};
        }
    }
}

void launch_expand_tables(cudaStream_t s, const DevRecipe *recipes, int nrec, u64 total_entries, int enc) {
    if (nrec < 1 || total_entries == 0) {
        return;
    }
    k_expand_tables<<<grid_for(total_entries, 256, 8), 256, 0, s>>>(recipes, nrec, total_entries, enc);
    cuda_check(cudaGetLastError(), "k_expand_tables launch");
    note_launch();
}

template <class T> __global__ void k_batch_set_one(cx<T> *const *__restrict__ svs, int n) {
    const int i = static_cast<int>(blockIdx.x * blockDim.x + threadIdx.x);
    if (i < n) {
        svs[i][0] = cx<T>{1, 0};
    }
}
template <class T> void launch_batch_set_one(cudaStream_t s, cx<T> *const *svs, int n) {
    if (n < 1) {
        return;
    }
    k_batch_set_one<T><<<(n + 255) / 256, 256, 0, s>>>(svs, n);
    cuda_check(cudaGetLastError(), "k_batch_set_one launch");
    note_launch();
}

namespace {

constexpr int kBatchRedThreads = 256;

template <class T> __device__ __forceinline__ cx<double> ld_amp(const cx<T> *a, u64 j, int dfm) {
    if constexpr (std::is_same_v<T, double>) {
        if (dfm) {
            const cx<df> v = reinterpret_cast<const cx<df> *>(a)[j];
            return cx<double>{df_to_double(v.x), df_to_double(v.y)};
        }
    }
    const cx<T> v = a[j];
    return cx<double>{static_cast<double>(v.x), static_cast<double>(v.y)};
}

__device__ __forceinline__ double batch_term_pair(const PauliTerm &t, u64 j, u64 jp, double ar, double ai) {
    const double s = (__popcll(j & t.yz) & 1) ? -1.0 : 1.0;
    const double sp = (__popcll(jp & t.yz) & 1) ? -1.0 : 1.0;
    // real part of i^ny ((s' + s) ar + i (s' - s) ai)
    switch (t.ny4) {
    case 0: return (sp + s) * ar;
    case 1: return -(sp - s) * ai;
    case 2: return -(sp + s) * ar;
    default: return (sp - s) * ai;
    }
}

} // namespace

// Block b of item it covers work units [c0, c0 + kBatchRedChunk) with
// c0 = (b - block_begin) * kBatchRedChunk; the partial of every block lands
// in its own slot, summed later in a fixed order.
template <class T>
__global__ void __launch_bounds__(kBatchRedThreads)
    k_pauli_batch(const BatchRedItem<T> *__restrict__ items, int nitems, double *__restrict__ partials) {
    const u64 b = blockIdx.x;
    int lo = 0, hi = nitems - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (items[mid].block_begin <= b) {
            lo = mid;
        } else {
            hi = mid - 1;
        }
    }
    const BatchRedItem<T> &it = items[lo];
    const PauliGroup &g = *it.group;
    const cx<T> *a = it.sv;
    const u64 c0 = (b - it.block_begin) * kBatchRedChunk;
    const u64 c1 = c0 + kBatchRedChunk < it.work ? c0 + kBatchRedChunk : it.work;
    double v = 0.0;
    if (g.x == 0) {
        for (u64 j = c0 + threadIdx.x; j < c1; j += kBatchRedThreads) {
            const cx<double> p = ld_amp<T>(a, j, it.df);
            const double w = p.x * p.x + p.y * p.y;
            double f = 0.0;
            for (int t = 0; t < g.nterms; t++) {
                f += (__popcll(j & g.t[t].yz) & 1) ? -g.t[t].coeff : g.t[t].coeff;
            }
            v += w * f;
        }
    } else {
        for (u64 k = c0 + threadIdx.x; k < c1; k += kBatchRedThreads) {
            const u64 j = insert_zero(k, g.hb);
            const u64 jp = j ^ g.x;
            const cx<double> p = ld_amp<T>(a, j, it.df);
            const cx<double> q = ld_amp<T>(a, jp, it.df);
            const double ar = p.x * q.x + p.y * q.y;
            const double ai = p.x * q.y - p.y * q.x;
            double f = 0.0;
            for (int t = 0; t < g.nterms; t++) {
                f += g.t[t].coeff * batch_term_pair(g.t[t], j, jp, ar, ai);
            }
            v += f;
        }
    }
    __shared__ double sh[kBatchRedThreads / 32];
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) {
        v += __shfl_down_sync(0xffffffffu, v, d);
    }
    if ((threadIdx.x & 31u) == 0) {
        sh[threadIdx.x >> 5] = v;
    }
    __syncthreads();
    if (threadIdx.x < 32) {
        double x = threadIdx.x < kBatchRedThreads / 32 ? sh[threadIdx.x] : 0.0;
#pragma unroll
        for (int d = 16; d > 0; d >>= 1) {
            x += __shfl_down_sync(0xffffffffu, x, d);
        }
        if (threadIdx.x == 0) {
            partials[b] = x;
        }
    }
}

// One warp per item: its blocks' partials in a fixed order.
template <class T>
__global__ void k_pauli_batch_items(const BatchRedItem<T> *__restrict__ items, int nitems, u64 total_blocks,
                                    const double *__restrict__ partials, double *__restrict__ item_sums) {
    const int it = static_cast<int>((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    const int lane = static_cast<int>(threadIdx.x & 31u);
    if (it >= nitems) {
        return;
    }
    const u64 b0 = items[it].block_begin;
    const u64 b1 = it + 1 < nitems ? items[it + 1].block_begin : total_blocks;
    double x = 0.0;
    for (u64 b = b0 + static_cast<u64>(lane); b < b1; b += 32) {
        x += partials[b];
    }
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) {
        x += __shfl_down_sync(0xffffffffu, x, d);
    }
    if (lane == 0) {
        item_sums[it] = x;
    }
}

template <class T>
void launch_pauli_batch(cudaStream_t s, const BatchRedItem<T> *items, int nitems, u64 total_blocks, double *partials,
                        double *item_sums) {
    if (nitems < 1) {
        return;
    }
    if (total_blocks > 0x7fffffffULL) {
        throw std::runtime_error("batched reduction: too many blocks");
    }
    k_pauli_batch<T><<<static_cast<unsigned>(total_blocks), kBatchRedThreads, 0, s>>>(items, nitems, partials);
    cuda_check(cudaGetLastError(), "k_pauli_batch launch");
    note_launch();
    const unsigned warps_per_block = 8;
    const unsigned grid = static_cast<unsigned>((static_cast<unsigned>(nitems) + warps_per_block - 1) / warps_per_block);
    k_pauli_batch_items<T><<<grid, 32 * warps_per_block, 0, s>>>(items, nitems, total_blocks, partials, item_sums);
    cuda_check(cudaGetLastError(), "k_pauli_batch_items launch");
    note_launch();
}

#define PLGB_BATCH_INST(T)                                                                                        \
    template void launch_tile_reg_batch<T>(cudaStream_t, int, const BatchTileItem<T> *, int, u64, int);          \
    template void launch_batch_set_one<T>(cudaStream_t, cx<T> *const *, int);                                    \
    template void launch_pauli_batch<T>(cudaStream_t, const BatchRedItem<T> *, int, u64, double *, double *);
PLGB_BATCH_INST(float)
PLGB_BATCH_INST(double)
template void launch_tile_reg_batch<df>(cudaStream_t, int, const BatchTileItem<df> *, int, u64, int);
template void launch_batch_set_one<df>(cudaStream_t, cx<df> *const *, int);

} // namespace plgb
