// Shared-memory tile passes: the per-op code shared by the single-register
// kernel (kernels_fused.cu) and the two-register adjoint kernel
// (kernels_adjoint.cu).  A tile of 2^t amplitudes sits in shared memory;
// every op of the pass runs on it with all threads of the CTA.
#pragma once

#include "df.cuh"
#include "fused.hpp"

namespace plgb {

namespace {

// local index j -> offset within the global index
__device__ __forceinline__ u64 local_offset(u32 j, const TilePassDesc &d) {
    u64 off = j & ((1u << d.L) - 1u);
#pragma unroll 4
    for (int m = 0; m < d.H; m++) {
        off |= static_cast<u64>((j >> (d.L + m)) & 1u) << d.hb[m];
    }
    return off;
}

__device__ __forceinline__ u32 insert_zeros32(u32 k, const int *ins, int nins) {
    for (int i = 0; i < nins; i++) {
        const int p = ins[i];
        const u32 lo = k & ((1u << p) - 1u);
        k = ((k >> p) << (p + 1)) | lo;
    }
    return k;
}

// sign flip on the integer pipe (no floating-point instruction)
__device__ __forceinline__ double flip_sign(double x, unsigned neg) {
    return __longlong_as_double(__double_as_longlong(x) ^ (static_cast<long long>(neg) << 63));
}
__device__ __forceinline__ float flip_sign(float x, unsigned neg) {
    return __int_as_float(__float_as_int(x) ^ static_cast<int>(neg << 31));
}
__device__ __forceinline__ df flip_sign(df x, unsigned neg) { return df{flip_sign(x.hi, neg), flip_sign(x.lo, neg)}; }
template <class T> __device__ __forceinline__ cx<T> flip(cx<T> v, unsigned neg) {
    return cx<T>{flip_sign(v.x, neg), flip_sign(v.y, neg)};
}
__device__ __forceinline__ float shfl_one(float x, int m) { return __shfl_xor_sync(0xffffffffu, x, m); }
__device__ __forceinline__ double shfl_one(double x, int m) { return __shfl_xor_sync(0xffffffffu, x, m); }
__device__ __forceinline__ df shfl_one(df x, int m) { return df{shfl_one(x.hi, m), shfl_one(x.lo, m)}; }
template <class T> __device__ __forceinline__ cx<T> shfl_xor(cx<T> v, int m) {
    return cx<T>{shfl_one(v.x, m), shfl_one(v.y, m)};
}

// Evaluate a small diagonal form on the global bits of a tile base.
template <class T> __device__ cx<T> form_value(const DiagForm<T> &f, u64 gbase) {
    unsigned k = 0;
    for (int b = 0; b < f.nb; b++) {
        k = (k << 1) | static_cast<unsigned>((gbase >> f.bits[b]) & 1u);
    }
    return f.tab[k];
}

// Tile-uniform state of the pass: the factor applied at the store and the
// parts of the last merged diagonal evaluated on the tile's global bits.
template <class T> struct SmemDiag {
    cx<T> tile_factor;
    u32 sign_mask;
    int ngen;
    int gen_bit[kMaxMixedForms];
    cx<T> gen_d0[kMaxMixedForms], gen_d1[kMaxMixedForms];
};

// Warp 0 evaluates the tile-uniform parts of a merged diagonal: the product
// of the global-bit factors, and per cross-boundary two-bit factor either a
// scalar, a sign flip of one local bit, or a general one-bit local factor.
// The caller synchronises before smem_apply.
template <class T>
__device__ __forceinline__ void smem_diag_prepare(const TileOp<T> &op, u64 gbase, const DiagForm<T> *__restrict__ forms,
                                                  SmemDiag<T> &sd) {
    if (threadIdx.x < 32) {
        const int lane = threadIdx.x;
        cx<T> sc{1, 0};
        for (int f = lane; f < op.ngforms; f += 32) {
            sc = sc * form_value<T>(forms[op.gform_begin + f], gbase);
        }
        u32 zl = 0;
        bool gen = false;
        cx<T> d0{1, 0}, d1{1, 0};
        int lb = 0;
        if (lane < op.nmforms) {
            const DiagForm<T> &mf = forms[op.mform_begin + lane];
            const unsigned gb = static_cast<unsigned>((gbase >> mf.bits[0]) & 1u);
            d0 = mf.tab[2 * gb];
            d1 = mf.tab[2 * gb + 1];
            lb = mf.local_bit;
            if (d1.x == d0.x && d1.y == d0.y) {
                sc = sc * d0;
            } else if (d1.x == -d0.x && d1.y == -d0.y) {
                sc = sc * d0;
                zl = 1u << lb;
            } else {
                gen = true;
            }
        }
#pragma unroll
        for (int m = 16; m > 0; m >>= 1) {
            sc = sc * shfl_xor(sc, m);
            zl ^= __shfl_xor_sync(0xffffffffu, zl, m);
        }
        const unsigned genmask = __ballot_sync(0xffffffffu, gen);
        if (gen) {
            const int slot = __popc(genmask & ((1u << lane) - 1u));
            sd.gen_bit[slot] = lb;
            sd.gen_d0[slot] = d0;
            sd.gen_d1[slot] = d1;
        }
        if (lane == 0) {
            sd.tile_factor = sd.tile_factor * sc;
            sd.sign_mask = zl;
            sd.ngen = __popc(genmask);
        }
    }
}

// Apply one op to the tile at `tile` (all threads; no barrier inside).
template <class T>
__device__ __forceinline__ void smem_apply(cx<T> *tile, const TileOp<T> &op, const TilePassDesc &d, u64 gbase,
                                           const cx<T> *__restrict__ tables, const SmemDiag<T> &sd) {
    const u32 T_ = 1u << d.t;
    switch (op.kind) {
    case TK_PAIR:
    case TK_SROT: {
        const u32 np = T_ >> op.nlins;
        for (u32 p = threadIdx.x; p < np; p += blockDim.x) {
            const u32 j0 = insert_zeros32(p, op.lins, op.nlins) | op.lcval;
            cx<T> &x = tile[j0 | op.lo0];
            cx<T> &y = tile[j0 | op.lo1];
            const cx<T> v0 = x, v1 = y;
            cx<T> r0, r1;
            if (op.kind == TK_SROT) {
                // [[a, -b], [b, a]] with one of a, b exactly 1
                const T ca = op.m[0].x, cb = op.m[0].y;
                if (op.mode == 0) { // a = 1, b = cb
                    r0 = cx<T>{v0.x - cb * v1.x, v0.y - cb * v1.y};
                    r1 = cx<T>{cb * v0.x + v1.x, cb * v0.y + v1.y};
                } else { // a = ca, b = 1
                    r0 = cx<T>{ca * v0.x - v1.x, ca * v0.y - v1.y};
                    r1 = cx<T>{v0.x + ca * v1.x, v0.y + ca * v1.y};
                }
            } else {
                switch (op.mode) {
                case M1_DENSE:
                    r0 = cfma(op.m[1], v1, op.m[0] * v0);
                    r1 = cfma(op.m[3], v1, op.m[2] * v0);
                    break;
                case M1_REAL:
                    r0 = cx<T>{op.m[0].x * v0.x + op.m[1].x * v1.x, op.m[0].x * v0.y + op.m[1].x * v1.y};
                    r1 = cx<T>{op.m[2].x * v0.x + op.m[3].x * v1.x, op.m[2].x * v0.y + op.m[3].x * v1.y};
                    break;
                case M1_RXF: {
                    const T c = op.m[0].x, s = op.m[1].y;
                    r0 = cx<T>{c * v0.x - s * v1.y, c * v0.y + s * v1.x};
                    r1 = cx<T>{c * v1.x - s * v0.y, c * v1.y + s * v0.x};
                    break;
                }
                case M1_DIAG:
                    r0 = op.m[0] * v0;
                    r1 = op.m[3] * v1;
                    break;
                case M1_PHASE1:
                    r0 = v0;
                    r1 = op.m[3] * v1;
                    break;
                case M1_SWAP:
                    r0 = v1;
                    r1 = v0;
                    break;
                case M1_ANTI:
                    r0 = op.m[1] * v1;
                    r1 = op.m[2] * v0;
                    break;
                default: // M1_NEG1
                    r0 = v0;
                    r1 = cx<T>{-v1.x, -v1.y};
                    break;
                }
            }
            x = r0;
            y = r1;
        }
        break;
    }
    case TK_DENSE2: {
        const u32 nq = T_ >> op.nlins;
        for (u32 p = threadIdx.x; p < nq; p += blockDim.x) {
            const u32 j0 = insert_zeros32(p, op.lins, op.nlins) | op.lcval;
            const u32 ix[4] = {j0, j0 | op.lo1, j0 | op.lo0, j0 | op.lo0 | op.lo1};
            cx<T> v[4];
#pragma unroll
            for (int r = 0; r < 4; r++) {
                v[r] = tile[ix[r]];
            }
#pragma unroll
            for (int r = 0; r < 4; r++) {
                cx<T> acc = op.m[4 * r] * v[0];
                acc = cfma(op.m[4 * r + 1], v[1], acc);
                acc = cfma(op.m[4 * r + 2], v[2], acc);
                acc = cfma(op.m[4 * r + 3], v[3], acc);
                tile[ix[r]] = acc;
            }
        }
        break;
    }
    case TK_DIAGTAB: {
        const u32 zl = sd.sign_mask;
        const int ngen = sd.ngen;
        const cx<T> *tab = tables + op.table_off;
        for (u32 j = threadIdx.x; j < T_; j += blockDim.x) {
            cx<T> v = op.has_table ? tab[j] * tile[j] : tile[j];
            for (int f = 0; f < ngen; f++) {
                v = (((j >> sd.gen_bit[f]) & 1u) ? sd.gen_d1[f] : sd.gen_d0[f]) * v;
            }
            tile[j] = flip(v, static_cast<unsigned>(__popc(j & zl) & 1));
        }
        break;
    }
    case TK_PARITY: {
        // a[i] *= s[popcount(i & pmask) & 1] where (i & cmask) == cval
        for (u32 j = threadIdx.x; j < T_; j += blockDim.x) {
            const u64 idx = gbase | local_offset(j, d);
            if ((idx & op.cmask) != op.cval) {
                if (op.zero_outside) {
                    tile[j] = cx<T>{0, 0};
                }
                continue;
            }
            tile[j] = ((__popcll(idx & op.pmask) & 1) ? op.m[1] : op.m[0]) * tile[j];
        }
        break;
    }
    default:
        break;
    }
}

} // namespace

} // namespace plgb
