// Fused adjoint sweep (host_adjoint.cpp): one tile pass applied to two
// registers at once, lambda and H lambda, with the parameter-derivative
// reductions evaluated inside the pass.
//
// The reverse sweep of AdjointJacobianLQubit.hpp:225-491 alternates, per
// operation, "Im <H lambda| G |lambda>" (when the operation is trainable)
// and "apply U^dagger to both registers".  Compiled as one program, the
// reductions become TK_REDUCE ops: a CTA holds the same tile of both
// registers in shared memory, applies the pass's ops to both, and at each
// reduction point adds the tile's share of Im <b| P G |a> (G a Pauli word on
// bits the pass keeps local, P a projector) to a per-CTA accumulator.  Each
// accumulator is written once per CTA into partials[slot * G + CTA]; a
// fixed-order sum over the G CTAs then gives the value, so results do not
// depend on timing.
//
// Deferred factors: the rotation scales and the tile-uniform diagonal
// factors of a pass are applied at the store.  Both registers receive the
// same ones, so at a reduction point they contribute |f|^2: the host stores
// the squared rotation scale so far (rmul), the kernel multiplies by
// |tile factor|^2.
#include "tile_smem.cuh"

#include <type_traits>

namespace plgb {

namespace {

constexpr int kAdjThreads = kTileThreads;

} // namespace

template <class T, class SI = T, class SO = T>
__global__ void __launch_bounds__(kAdjThreads)
    k_tile_adj(cx<SI> *a, cx<SI> *b, const TilePassDesc dp, const TileOp<T> *__restrict__ ops,
               const DiagForm<T> *__restrict__ forms, const cx<T> *__restrict__ tables, double *__restrict__ partials,
               int G) {
    extern __shared__ unsigned char smraw[];
    __shared__ SmemDiag<T> sd;
    __shared__ TilePassDesc d;
    __shared__ double s_acc[kMaxReducePerPass];
    __shared__ double s_red[kAdjThreads / 32];
    if (threadIdx.x == 0) {
        d = dp;
    }
    for (int i = threadIdx.x; i < kMaxReducePerPass; i += blockDim.x) {
        s_acc[i] = 0.0;
    }
    __syncthreads();
    const u32 T_ = 1u << d.t;
    cx<T> *ta = reinterpret_cast<cx<T> *>(smraw);
    cx<T> *tb = ta + T_;
    for (u64 g = blockIdx.x; g < d.ntiles; g += gridDim.x) {
        u64 gbase = g << d.L;
        for (int m = 0; m < d.H; m++) {
            const int p = d.hb[m];
            gbase = ((gbase >> p) << (p + 1)) | (gbase & ((u64{1} << p) - 1));
        }
        for (u32 j = threadIdx.x; j < T_; j += blockDim.x) {
            const u64 gj = gbase | local_offset(j, d);
            ta[j] = ld_conv<T, SI>(a[gj]);
            tb[j] = ld_conv<T, SI>(b[gj]);
        }
        if (threadIdx.x == 0) {
            sd.tile_factor = cx<T>{1, 0};
        }
        __syncthreads();
        for (int oi = 0; oi < d.nops; oi++) {
            const TileOp<T> &op = ops[d.op_begin + oi];
            if ((gbase & op.gcmask) != op.gcval) {
                continue;
            }
            if (op.kind == TK_REDUCE) {
                // Im sum_j [(j & P) == pv] conj(b_j) i^ny (-1)^|k & yz| a_k, k = j ^ x.
                // The projector's and the parity's global bits are tile-uniform
                // (the projector's gate the whole op, like global controls);
                // i^ny selects which of Re / Im of conj(b) a is needed.
                const unsigned gpar = static_cast<unsigned>(__popcll(gbase & op.pmask) & 1);
                const bool want_re = (op.mode & 1) != 0;
                const double sgn = (op.mode & 2) ? -1.0 : 1.0;
                double v = 0.0;
                if constexpr (std::is_same_v<T, df>) {
                    // double-float products and a double-float running sum,
                    // one conversion per thread
                    df acc{0.f, 0.f};
                    for (u32 j = threadIdx.x; j < T_; j += blockDim.x) {
                        if ((j & op.rcmask) != op.lcval) {
                            continue;
                        }
                        const u32 k = j ^ op.lo1;
                        const cx<df> p = tb[j];
                        const cx<df> q = ta[k];
                        df z = want_re ? p.x * q.x + p.y * q.y : p.x * q.y - p.y * q.x;
                        if ((static_cast<unsigned>(__popc(k & op.lo0)) ^ gpar) & 1u) {
                            z = -z;
                        }
                        acc = acc + z;
                    }
                    v = df_to_double(acc);
                } else {
                    for (u32 j = threadIdx.x; j < T_; j += blockDim.x) {
                        if ((j & op.rcmask) != op.lcval) {
                            continue;
                        }
                        const u32 k = j ^ op.lo1;
                        const cx<T> p = tb[j];
                        const cx<T> q = ta[k];
                        double z = want_re ? static_cast<double>(p.x) * q.x + static_cast<double>(p.y) * q.y
                                           : static_cast<double>(p.x) * q.y - static_cast<double>(p.y) * q.x;
                        if ((static_cast<unsigned>(__popc(k & op.lo0)) ^ gpar) & 1u) {
                            z = -z;
                        }
                        v += z;
                    }
                }
                v *= sgn;
#pragma unroll
                for (int m = 16; m > 0; m >>= 1) {
                    v += __shfl_down_sync(0xffffffffu, v, m);
                }
                if ((threadIdx.x & 31u) == 0) {
                    s_red[threadIdx.x >> 5] = v;
                }
                __syncthreads();
                if (threadIdx.x == 0) {
                    double tot = 0.0;
                    for (int w = 0; w < static_cast<int>(blockDim.x >> 5); w++) {
                        tot += s_red[w];
                    }
                    const cx<T> f = sd.tile_factor;
                    double fx, fy;
                    if constexpr (std::is_same_v<T, df>) {
                        fx = static_cast<double>(f.x);
                        fy = static_cast<double>(f.y);
                    } else {
                        fx = static_cast<double>(f.x);
                        fy = static_cast<double>(f.y);
                    }
                    const double f2 = fx * fx + fy * fy;
                    s_acc[op.diag_slot] += tot * op.rmul * f2;
                }
                __syncthreads();
                continue;
            }
            if (op.kind == TK_DIAGTAB) {
                smem_diag_prepare<T>(op, gbase, forms, sd);
                __syncthreads();
            }
            smem_apply<T>(ta, op, d, gbase, tables, sd);
            smem_apply<T>(tb, op, d, gbase, tables, sd);
            __syncthreads();
        }
        const cx<T> f = sd.tile_factor;
        const T ps = from_double<T>(d.pass_scale);
        const cx<T> sf{f.x * ps, f.y * ps};
        cx<SO> *ao = reinterpret_cast<cx<SO> *>(a);
        cx<SO> *bo = reinterpret_cast<cx<SO> *>(b);
        for (u32 j = threadIdx.x; j < T_; j += blockDim.x) {
            const u64 gj = gbase | local_offset(j, d);
            ao[gj] = st_conv<SO, T>(sf * ta[j]);
            bo[gj] = st_conv<SO, T>(sf * tb[j]);
        }
        __syncthreads();
    }
    // one write per reduction op of the pass and CTA (every slot belongs to
    // exactly one pass; CTAs without tiles write their zero)
    for (int oi = threadIdx.x; oi < d.nops; oi += blockDim.x) {
        const TileOp<T> &op = ops[d.op_begin + oi];
        if (op.kind == TK_REDUCE && static_cast<int>(blockIdx.x) < G) {
            partials[static_cast<size_t>(op.rslot) * static_cast<size_t>(G) + blockIdx.x] = s_acc[op.diag_slot];
        }
    }
}

namespace {
template <class T, class SI = T, class SO = T> void adj_smem_attr() {
    static bool attr = false;
    if (!attr) {
        cuda_check(cudaFuncSetAttribute(k_tile_adj<T, SI, SO>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        200 * 1024), "adjoint tile smem attribute");
        attr = true;
    }
}
} // namespace

int adj_grid_capacity(size_t tile_bytes_each) {
    // the launcher's grid never exceeds this many CTAs for 2 tiles of this size
    adj_smem_attr<double>();
    adj_smem_attr<float>();
    adj_smem_attr<df, double, df>();
    adj_smem_attr<df, df, df>();
    adj_smem_attr<df, df, double>();
    adj_smem_attr<df, double, double>();
    int per_sm = 1;
    const size_t smem = 2 * tile_bytes_each;
    cuda_check(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_tile_adj<double>, kAdjThreads, smem),
               "adjoint occupancy");
    int per_sm_f = 1;
    cuda_check(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm_f, k_tile_adj<float>, kAdjThreads, smem),
               "adjoint occupancy");
    return LaunchGeom::sm_count() * std::max(1, std::max(per_sm, per_sm_f));
}

template <class T>
void launch_tile_pass_adj(cudaStream_t s, cx<T> *lam, cx<T> *hlam, const TilePassDesc &d, const TileOp<T> *ops,
                          const DiagForm<T> *forms, const cx<T> *tables, double *partials, int G) {
    const size_t smem = 2 * (sizeof(cx<T>) << d.t);
    adj_smem_attr<T>();
    if (smem > 200 * 1024) {
        throw std::runtime_error("adjoint tile pass: two tiles do not fit shared memory");
    }
    int per_sm = 1;
    cuda_check(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_tile_adj<T>, kAdjThreads, smem),
               "adjoint occupancy");
    if (per_sm < 1) {
        throw std::runtime_error("adjoint tile pass: tile does not fit one SM");
    }
    const u64 cap = static_cast<u64>(LaunchGeom::sm_count()) * static_cast<u64>(per_sm);
    u64 grid = d.ntiles < cap ? d.ntiles : cap;
    if (grid > static_cast<u64>(G)) {
        grid = static_cast<u64>(G);
    }
    k_tile_adj<T><<<static_cast<unsigned>(grid), kAdjThreads, smem, s>>>(lam, hlam, d, ops, forms, tables, partials, G);
    cuda_check(cudaGetLastError(), "k_tile_adj launch");
    note_launch();
}

template <class SI, class SO>
static void launch_adj_df_io(cudaStream_t s, void *lam, void *hlam, const TilePassDesc &d, const TileOp<df> *ops,
                             const DiagForm<df> *forms, const cx<df> *tables, double *partials, int G) {
    const size_t smem = 2 * (sizeof(cx<df>) << d.t);
    adj_smem_attr<df, SI, SO>();
    if (smem > 200 * 1024) {
        throw std::runtime_error("adjoint tile pass: two tiles do not fit shared memory");
    }
    int per_sm = 1;
    cuda_check(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_tile_adj<df, SI, SO>, kAdjThreads, smem),
               "adjoint occupancy");
    if (per_sm < 1) {
        throw std::runtime_error("adjoint tile pass: tile does not fit one SM");
    }
    const u64 cap = static_cast<u64>(LaunchGeom::sm_count()) * static_cast<u64>(per_sm);
    u64 grid = d.ntiles < cap ? d.ntiles : cap;
    if (grid > static_cast<u64>(G)) {
        grid = static_cast<u64>(G);
    }
    k_tile_adj<df, SI, SO><<<static_cast<unsigned>(grid), kAdjThreads, smem, s>>>(
        static_cast<cx<SI> *>(lam), static_cast<cx<SI> *>(hlam), d, ops, forms, tables, partials, G);
    cuda_check(cudaGetLastError(), "k_tile_adj (df) launch");
    note_launch();
}

void launch_tile_pass_adj_df(cudaStream_t s, void *lam, void *hlam, int io, const TilePassDesc &d,
                             const TileOp<df> *ops, const DiagForm<df> *forms, const cx<df> *tables, double *partials,
                             int G) {
    switch (io) {
    case 0: launch_adj_df_io<double, double>(s, lam, hlam, d, ops, forms, tables, partials, G); break;
    case 1: launch_adj_df_io<double, df>(s, lam, hlam, d, ops, forms, tables, partials, G); break;
    case 2: launch_adj_df_io<df, df>(s, lam, hlam, d, ops, forms, tables, partials, G); break;
    default: launch_adj_df_io<df, double>(s, lam, hlam, d, ops, forms, tables, partials, G); break;
    }
}

// out[slot] = sum over CTAs of partials[slot * G + c], one warp per slot in a
// fixed order
__global__ void k_adj_sum(const double *__restrict__ partials, int nslots, int G, double *__restrict__ out) {
    const int slot = static_cast<int>((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    const int lane = static_cast<int>(threadIdx.x & 31u);
    if (slot >= nslots) {
        return;
    }
    double x = 0.0;
    for (int c = lane; c < G; c += 32) {
        x += partials[static_cast<size_t>(slot) * static_cast<size_t>(G) + c];
    }
#pragma unroll
    for (int m = 16; m > 0; m >>= 1) {
        x += __shfl_down_sync(0xffffffffu, x, m);
    }
    if (lane == 0) {
        out[slot] = x;
    }
}

void launch_adj_sum(cudaStream_t s, const double *partials, int nslots, int G, double *out) {
    if (nslots < 1) {
        return;
    }
    const unsigned grid = static_cast<unsigned>((nslots + 7) / 8);
    k_adj_sum<<<grid, 256, 0, s>>>(partials, nslots, G, out);
    cuda_check(cudaGetLastError(), "k_adj_sum launch");
    note_launch();
}

template void launch_tile_pass_adj<float>(cudaStream_t, cx<float> *, cx<float> *, const TilePassDesc &,
                                          const TileOp<float> *, const DiagForm<float> *, const cx<float> *, double *,
                                          int);
template void launch_tile_pass_adj<double>(cudaStream_t, cx<double> *, cx<double> *, const TilePassDesc &,
                                           const TileOp<double> *, const DiagForm<double> *, const cx<double> *,
                                           double *, int);

} // namespace plgb
