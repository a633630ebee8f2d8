// Register-blocked fused tile passes (sm_103a).
//
// Same pass semantics as kernels_fused.cu, different execution: a CTA of
// 2^(t-4) threads holds its tile of 2^t amplitudes in registers, 16 per
// thread.  The host splits the pass into stages.  In a register stage four
// local bits are "register bits" (amplitudes differing only in them live in
// the same thread) and every one-target op on them is pure register
// arithmetic: no shared memory, no index math, no barrier.  Changing the
// register bits is one shared-memory transpose (XOR-swizzled so that strided
// thread patterns stay conflict-free).  Two-target ops run in a shared-memory
// stage.  Merged diagonals are evaluated per tile once, in a prologue, and
// applied in registers from the per-pass table.
#include "tile_reg.cuh"

#include <atomic>

namespace plgb {

// OCC: launch bounds that cap registers at 128 per thread (16 warps per SM
// for 2^11-amplitude tiles instead of 8), trading some spills for latency
// hiding; chosen per precision (tile_variant_occ).
#define PLGB_TILE_BOUNDS(OCC) __launch_bounds__(256, (OCC) ? 2 : 1)

// op records staged in shared memory for complex64 only (fewer spills at 128
// registers for complex128 and double-float when read from global memory)
template <class T> constexpr bool kStageRecs = std::is_same_v<T, float>;

template <class T, bool OCC>
__global__ void PLGB_TILE_BOUNDS(OCC) k_tile_reg(cx<T> *__restrict__ a, const TilePassDesc d,
                                                 const TileOp<T> *__restrict__ ops,
                                                 const DiagForm<T> *__restrict__ forms,
                                                 const cx<T> *__restrict__ tables,
                                                 const StageDesc *__restrict__ stages) {
    extern __shared__ unsigned char smraw[];
    cx<T> *tile = reinterpret_cast<cx<T> *>(smraw);
    __shared__ TileShared<T> sh;
    // the descriptor is indexed dynamically (hb[]): keep it in shared memory
    __shared__ TilePassDesc sd;
    if (threadIdx.x == 0) {
        sd = d;
    }
    const auto *recs = op_records<T, kStageRecs<T>>(smraw + (sizeof(cx<T>) << d.t), ops, d);
    __syncthreads();
    for (u64 g = blockIdx.x; g < sd.ntiles; g += gridDim.x) {
        tile_reg_run<T>(a, a, sd, ops, forms, tables, stages, g, tile, sh, recs);
    }
}

template <class SI, class SO, bool OCC>
__global__ void PLGB_TILE_BOUNDS(OCC) k_tile_reg_df(const cx<SI> *ain, cx<SO> *aout, const TilePassDesc d,
                                                    const TileOp<df> *__restrict__ ops,
                                                    const DiagForm<df> *__restrict__ forms,
                                                    const cx<df> *__restrict__ tables,
                                                    const StageDesc *__restrict__ stages) {
    extern __shared__ unsigned char smraw[];
    cx<df> *tile = reinterpret_cast<cx<df> *>(smraw);
    __shared__ TileShared<df> sh;
    __shared__ TilePassDesc sd;
    if (threadIdx.x == 0) {
        sd = d;
    }
    const auto *recs = op_records<df, kStageRecs<df>>(smraw + (sizeof(cx<df>) << d.t), ops, d);
    __syncthreads();
    for (u64 g = blockIdx.x; g < sd.ntiles; g += gridDim.x) {
        tile_reg_run<df, SI, SO>(ain, aout, sd, ops, forms, tables, stages, g, tile, sh, recs);
    }
}

namespace {
std::atomic<int> g_occ_c64{1}, g_occ_c128{1}; // measured faster on GB300 for both
} // namespace
bool tile_variant_occ(int precision) { return (precision == 128 ? g_occ_c128 : g_occ_c64).load() != 0; }
bool set_tile_variant_occ(int precision, bool occ) {
    return (precision == 128 ? g_occ_c128 : g_occ_c64).exchange(occ ? 1 : 0) != 0;
}

// persistent grid: SMs x resident CTAs of this kernel and tile size
template <class K> static unsigned tile_grid(K kernel, int threads, size_t smem, u64 ntiles, bool &attr) {
    if (!attr) {
        cuda_check(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024),
                   "tile smem attribute");
        attr = true;
    }
    int per_sm = 1;
    cuda_check(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, smem), "occupancy");
    if (per_sm < 1) {
        throw std::runtime_error("register tile pass: tile does not fit one SM");
    }
    const u64 cap = static_cast<u64>(LaunchGeom::sm_count()) * static_cast<u64>(per_sm);
    return static_cast<unsigned>(ntiles < cap ? ntiles : cap);
}

template <class SI, class SO, bool OCC>
static void launch_df(cudaStream_t s, void *sv, const TilePassDesc &d, const TileOp<df> *ops, const DiagForm<df> *forms,
                      const cx<df> *tables, const StageDesc *stages) {
    const int threads = 1 << (d.t - kRegBits);
    const size_t smem = (sizeof(cx<df>) << d.t) + op_record_bytes<df, kStageRecs<df>>(d.nops);
    static bool attr = false;
    const unsigned grid = tile_grid(k_tile_reg_df<SI, SO, OCC>, threads, smem, d.ntiles, attr);
    k_tile_reg_df<SI, SO, OCC><<<grid, threads, smem, s>>>(static_cast<const cx<SI> *>(sv), static_cast<cx<SO> *>(sv),
                                                           d, ops, forms, tables, stages);
    cuda_check(cudaGetLastError(), "k_tile_reg_df launch");
    note_launch();
}

template <bool OCC>
static void launch_df_io(cudaStream_t s, void *sv, int io, const TilePassDesc &d, const TileOp<df> *ops,
                         const DiagForm<df> *forms, const cx<df> *tables, const StageDesc *stages) {
    switch (io) {
    case 0: launch_df<double, double, OCC>(s, sv, d, ops, forms, tables, stages); break;
    case 1: launch_df<double, df, OCC>(s, sv, d, ops, forms, tables, stages); break;
    case 2: launch_df<df, df, OCC>(s, sv, d, ops, forms, tables, stages); break;
    default: launch_df<df, double, OCC>(s, sv, d, ops, forms, tables, stages); break;
    }
}

void launch_tile_pass_reg_df(cudaStream_t s, void *sv, int io, const TilePassDesc &d, const TileOp<df> *ops,
                             const DiagForm<df> *forms, const cx<df> *tables, const StageDesc *stages) {
    if (d.t < kMinRegTileBits || d.t > 12 || d.ndiag > kMaxDiagOpsPerPass || d.nops > kMaxOpsPerPass) {
        throw std::runtime_error("register tile pass (df): unsupported geometry");
    }
    if (tile_variant_occ(128)) {
        launch_df_io<true>(s, sv, io, d, ops, forms, tables, stages);
    } else {
        launch_df_io<false>(s, sv, io, d, ops, forms, tables, stages);
    }
}

template <class T, bool OCC>
static void launch_reg(cudaStream_t s, cx<T> *sv, const TilePassDesc &d, const TileOp<T> *ops, const DiagForm<T> *forms,
                       const cx<T> *tables, const StageDesc *stages) {
    const int threads = 1 << (d.t - kRegBits);
    const size_t smem = (sizeof(cx<T>) << d.t) + op_record_bytes<T, kStageRecs<T>>(d.nops);
    static bool attr = false;
    const unsigned grid = tile_grid(k_tile_reg<T, OCC>, threads, smem, d.ntiles, attr);
    k_tile_reg<T, OCC><<<grid, threads, smem, s>>>(sv, d, ops, forms, tables, stages);
    cuda_check(cudaGetLastError(), "k_tile_reg launch");
    note_launch();
}

template <class T>
void launch_tile_pass_reg(cudaStream_t s, cx<T> *sv, const TilePassDesc &d, const TileOp<T> *ops,
                          const DiagForm<T> *forms, const cx<T> *tables, const StageDesc *stages) {
    if (d.t < kMinRegTileBits || d.t > 12 || d.ndiag > kMaxDiagOpsPerPass || d.nops > kMaxOpsPerPass) {
        throw std::runtime_error("register tile pass: unsupported geometry");
    }
    if (tile_variant_occ(sizeof(T) == 8 ? 128 : 64)) {
        launch_reg<T, true>(s, sv, d, ops, forms, tables, stages);
    } else {
        launch_reg<T, false>(s, sv, d, ops, forms, tables, stages);
    }
}

template void launch_tile_pass_reg<float>(cudaStream_t, cx<float> *, const TilePassDesc &, const TileOp<float> *,
                                          const DiagForm<float> *, const cx<float> *, const StageDesc *);
template void launch_tile_pass_reg<double>(cudaStream_t, cx<double> *, const TilePassDesc &, const TileOp<double> *,
                                           const DiagForm<double> *, const cx<double> *, const StageDesc *);

} // namespace plgb
