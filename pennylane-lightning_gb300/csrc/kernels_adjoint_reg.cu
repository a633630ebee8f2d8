// Fused adjoint sweep on the register-blocked tile kernel (sm_103a).
//
// Same pass semantics as k_tile_adj (kernels_adjoint.cu): every op of the
// reverse program is applied to both lambda and H lambda, and each TK_REDUCE
// op adds Im <H lambda| P G |lambda> over the tile to its parameter slot.
// Here the CTA holds the same tile of both registers in registers (8
// amplitudes of each per thread: 3 register bits, tile_reg_run with DUAL and
// 2^(t-3) threads, so a thread keeps as many amplitudes as in the
// single-register kernel): the planner puts
// every reduction in a register stage whose register bits hold its flip
// bit, so both amplitudes of each summed pair sit in one thread.  A
// reduction's share is summed per thread, then per warp by shuffles, and
// accumulated into a per-warp shared slot across the CTA's tiles; the slots
// are added in warp order at the end and written once per CTA, so results do
// not depend on timing.
#include "tile_reg.cuh"

namespace plgb {

template <class T, class SI, class SO>
__global__ void __launch_bounds__(512, 1)
    k_tile_reg_adj(cx<SI> *a, cx<SI> *b, const TilePassDesc d, const TileOp<T> *__restrict__ ops,
                   const DiagForm<T> *__restrict__ forms, const cx<T> *__restrict__ tables,
                   const StageDesc *__restrict__ stages, double *__restrict__ partials, int G) {
    extern __shared__ unsigned char smraw[];
    cx<T> *tile = reinterpret_cast<cx<T> *>(smraw);
    cx<T> *tileb = tile + (size_t{1} << d.t);
    __shared__ TileShared<T> sh;
    __shared__ TilePassDesc sd;
    __shared__ double s_part[kMaxReducePerPass * 16];
    __shared__ double s_f2[kMaxDiagOpsPerPass + 1];
    if (threadIdx.x == 0) {
        sd = d;
    }
    for (int i = static_cast<int>(threadIdx.x); i < kMaxReducePerPass * 16; i += static_cast<int>(blockDim.x)) {
        s_part[i] = 0.0;
    }
    __syncthreads();
    const TileOp<T> *recs = ops + d.op_begin;
    for (u64 g = blockIdx.x; g < sd.ntiles; g += gridDim.x) {
        tile_reg_run<T, SI, SO, true, kAdjRegBits>(a, reinterpret_cast<cx<SO> *>(a), sd, ops, forms, tables, stages, g, tile, sh,
                                      recs, b, reinterpret_cast<cx<SO> *>(b), tileb, s_part, s_f2);
    }
    __syncthreads();
    const int nwarps = static_cast<int>(blockDim.x >> 5);
    for (int oi = static_cast<int>(threadIdx.x); oi < sd.nops; oi += static_cast<int>(blockDim.x)) {
        const TileOp<T> &op = ops[sd.op_begin + oi];
        if (op.kind == TK_REDUCE && static_cast<int>(blockIdx.x) < G) {
            double tot = 0.0;
            for (int w = 0; w < nwarps; w++) {
                tot += s_part[op.diag_slot * nwarps + w];
            }
            partials[static_cast<size_t>(op.rslot) * static_cast<size_t>(G) + blockIdx.x] = tot;
        }
    }
}

namespace {

template <class T, class SI, class SO>
void launch_reg_adj(cudaStream_t s, void *lam, void *hlam, const TilePassDesc &d, const TileOp<T> *ops,
                    const DiagForm<T> *forms, const cx<T> *tables, const StageDesc *stages, double *partials,
                    int G) {
    if (d.t < kMinRegTileBits || d.t > 12 || d.ndiag > kMaxDiagOpsPerPass || d.nops > kMaxOpsPerPass ||
        d.nrslots > kMaxReducePerPass || G < 1) {
        throw std::runtime_error("register adjoint pass: unsupported geometry");
    }
    const int threads = 1 << (d.t - kAdjRegBits);
    const size_t smem = 2 * (sizeof(cx<T>) << d.t);
    static bool attr = false;
    if (!attr) {
        cuda_check(cudaFuncSetAttribute(k_tile_reg_adj<T, SI, SO>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        200 * 1024),
                   "register adjoint smem attribute");
        attr = true;
    }
    int per_sm = 1;
    cuda_check(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_tile_reg_adj<T, SI, SO>, threads, smem),
               "register adjoint occupancy");
    if (per_sm < 1) {
        throw std::runtime_error("register adjoint pass: two tiles do not fit one SM");
    }
    const u64 cap = static_cast<u64>(LaunchGeom::sm_count()) * static_cast<u64>(per_sm);
    u64 grid = d.ntiles < cap ? d.ntiles : cap;
    if (grid > static_cast<u64>(G)) {
        grid = static_cast<u64>(G);
    }
    k_tile_reg_adj<T, SI, SO><<<static_cast<unsigned>(grid), threads, smem, s>>>(
        static_cast<cx<SI> *>(lam), static_cast<cx<SI> *>(hlam), d, ops, forms, tables, stages, partials, G);
    cuda_check(cudaGetLastError(), "k_tile_reg_adj launch");
    note_launch();
}

} // namespace

template <class T>
void launch_tile_pass_reg_adj(cudaStream_t s, cx<T> *lam, cx<T> *hlam, const TilePassDesc &d, const TileOp<T> *ops,
                              const DiagForm<T> *forms, const cx<T> *tables, const StageDesc *stages,
                              double *partials, int G) {
    launch_reg_adj<T, T, T>(s, lam, hlam, d, ops, forms, tables, stages, partials, G);
}

void launch_tile_pass_reg_adj_df(cudaStream_t s, void *lam, void *hlam, int io, const TilePassDesc &d,
                                 const TileOp<df> *ops, const DiagForm<df> *forms, const cx<df> *tables,
                                 const StageDesc *stages, double *partials, int G) {
    switch (io) {
    case 0: launch_reg_adj<df, double, double>(s, lam, hlam, d, ops, forms, tables, stages, partials, G); break;
    case 1: launch_reg_adj<df, double, df>(s, lam, hlam, d, ops, forms, tables, stages, partials, G); break;
    case 2: launch_reg_adj<df, df, df>(s, lam, hlam, d, ops, forms, tables, stages, partials, G); break;
    default: launch_reg_adj<df, df, double>(s, lam, hlam, d, ops, forms, tables, stages, partials, G); break;
    }
}

template void launch_tile_pass_reg_adj<float>(cudaStream_t, cx<float> *, cx<float> *, const TilePassDesc &,
                                              const TileOp<float> *, const DiagForm<float> *, const cx<float> *,
                                              const StageDesc *, double *, int);
template void launch_tile_pass_reg_adj<double>(cudaStream_t, cx<double> *, cx<double> *, const TilePassDesc &,
                                               const TileOp<double> *, const DiagForm<double> *,
                                               const cx<double> *, const StageDesc *, double *, int);

} // namespace plgb
