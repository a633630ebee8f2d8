// Register-blocked fused tile pass: the per-tile body shared by the
// single-register kernel (kernels_fused_reg.cu) and the batched kernel over
// many registers (kernels_batch.cu).
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
#pragma once

#include <type_traits>

#include "df.cuh"
#include "fused.hpp"

namespace plgb {

namespace {


template <class T> __device__ __forceinline__ u32 swz(u32 j) {
    if constexpr (sizeof(T) == 8) { // 16-byte amplitudes: 8 per 128-byte row
        return j ^ (((j >> 3) ^ (j >> 6) ^ (j >> 9) ^ (j >> 12)) & 7u);
    } else { // 8-byte amplitudes: 16 per row
        return j ^ (((j >> 4) ^ (j >> 8) ^ (j >> 12)) & 15u);
    }
}

__device__ __forceinline__ u64 local_offset_r(u32 j, const TilePassDesc &d) {
    u64 off = j & ((1u << d.L) - 1u);
#pragma unroll 4
    for (int m = 0; m < d.H; m++) {
        off |= static_cast<u64>((j >> (d.L + m)) & 1u) << d.hb[m];
    }
    return off;
}

__device__ __forceinline__ u32 insert_zeros_r(u32 k, const int *ins, int nins) {
    for (int i = 0; i < nins; i++) {
        const int p = ins[i];
        k = ((k >> p) << (p + 1)) | (k & ((1u << p) - 1u));
    }
    return k;
}

__device__ __forceinline__ double sflip(double x, unsigned neg) {
    return __longlong_as_double(__double_as_longlong(x) ^ (static_cast<long long>(neg) << 63));
}
__device__ __forceinline__ float sflip(float x, unsigned neg) {
    return __int_as_float(__float_as_int(x) ^ static_cast<int>(neg << 31));
}
__device__ __forceinline__ df sflip(df x, unsigned neg) { return df{sflip(x.hi, neg), sflip(x.lo, neg)}; }
template <class T> __device__ __forceinline__ cx<T> cflip(cx<T> v, unsigned neg) {
    return cx<T>{sflip(v.x, neg), sflip(v.y, neg)};
}
__device__ __forceinline__ float shfl_val(float x, int m) { return __shfl_xor_sync(0xffffffffu, x, m); }
__device__ __forceinline__ double shfl_val(double x, int m) { return __shfl_xor_sync(0xffffffffu, x, m); }
__device__ __forceinline__ df shfl_val(df x, int m) { return df{shfl_val(x.hi, m), shfl_val(x.lo, m)}; }
template <class T> __device__ __forceinline__ cx<T> shx(cx<T> v, int m) {
    return cx<T>{shfl_val(v.x, m), shfl_val(v.y, m)};
}


// State amplitudes stream through a pass once: load and store them with the
// evict-first cache policy so that they do not push the pass's diagonal
// tables and op records (read by every tile) out of L1.
__device__ __forceinline__ cx<float> ld_stream(const cx<float> *p) {
    const float2 t = __ldcs(reinterpret_cast<const float2 *>(p));
    return cx<float>{t.x, t.y};
}
__device__ __forceinline__ cx<double> ld_stream(const cx<double> *p) {
    const double2 t = __ldcs(reinterpret_cast<const double2 *>(p));
    return cx<double>{t.x, t.y};
}
__device__ __forceinline__ cx<df> ld_stream(const cx<df> *p) {
    const float4 t = __ldcs(reinterpret_cast<const float4 *>(p));
    return cx<df>{df{t.x, t.y}, df{t.z, t.w}};
}
__device__ __forceinline__ void st_stream(cx<float> *p, cx<float> v) {
    __stcs(reinterpret_cast<float2 *>(p), make_float2(v.x, v.y));
}
__device__ __forceinline__ void st_stream(cx<double> *p, cx<double> v) {
    __stcs(reinterpret_cast<double2 *>(p), make_double2(v.x, v.y));
}
__device__ __forceinline__ void st_stream(cx<df> *p, cx<df> v) {
    __stcs(reinterpret_cast<float4 *>(p), make_float4(v.x.hi, v.x.lo, v.y.hi, v.y.lo));
}

// Layout of a register stage, held in registers: local index of register
// slot i of this thread = jt | (bit k of i placed at local bit rb[k]).
// The canonical layout (load / store) has rb = {w, w+1, w+2, w+3}, jt = tid.
struct Layout {
    u32 jt;
    int rb0, rb1, rb2, rb3;
    __device__ __forceinline__ u32 reg(int i) const {
        return ((i & 1) ? (1u << rb0) : 0u) | ((i & 2) ? (1u << rb1) : 0u) | ((i & 4) ? (1u << rb2) : 0u) |
               ((i & 8) ? (1u << rb3) : 0u);
    }
    __device__ __forceinline__ u32 at(int i) const { return jt | reg(i); }
};
__device__ __forceinline__ Layout canonical_layout(u32 tid, int w) { return Layout{tid, w, w + 1, w + 2, w + 3}; }
__device__ __forceinline__ Layout stage_layout(const StageDesc *st, u32 tid, int w) {
    u32 jt = 0;
    for (int m = 0; m < w; m++) {
        jt |= ((tid >> m) & 1u) << st->tb[m];
    }
    return Layout{jt, st->rb[0], st->rb[1], st->rb[2], st->rb[3]};
}

// Shared-memory addresses of a thread's 16 slots.  The swizzle is linear
// over XOR and the thread and register parts of a local index have disjoint
// bits, so swz(jt | reg(i)) = swz(jt) ^ (XOR of swz(1 << rb_k) over the set
// bits k of i): four swizzles per layout, then one XOR per slot.
template <class T> struct SlotAddr {
    u32 base, s0, s1, s2, s3;
    __device__ __forceinline__ explicit SlotAddr(const Layout &l)
        : base(swz<T>(l.jt)), s0(swz<T>(1u << l.rb0)), s1(swz<T>(1u << l.rb1)), s2(swz<T>(1u << l.rb2)),
          s3(swz<T>(1u << l.rb3)) {}
    __device__ __forceinline__ u32 operator()(int i) const {
        return base ^ ((i & 1) ? s0 : 0u) ^ ((i & 2) ? s1 : 0u) ^ ((i & 4) ? s2 : 0u) ^ ((i & 8) ? s3 : 0u);
    }
};
template <class T, int N> __device__ __forceinline__ void to_smem(cx<T> *tile, const cx<T> (&v)[N], const Layout &l) {
    const SlotAddr<T> ad(l);
#pragma unroll
    for (int i = 0; i < N; i++) {
        tile[ad(i)] = v[i];
    }
}
template <class T, int N> __device__ __forceinline__ void from_smem(const cx<T> *tile, cx<T> (&v)[N], const Layout &l) {
    const SlotAddr<T> ad(l);
#pragma unroll
    for (int i = 0; i < N; i++) {
        v[i] = tile[ad(i)];
    }
}

// One-target op on register bit K for the pairs of a thread, one
// specialisation per op shape so the unrolled body has no mode branches.
// TWO: the same op on a second register array v2 (adjoint sweeps), sharing
// the coefficients and the control tests.
template <int MODE, bool CTRL, class T, int K, bool TWO, class OP, int N>
__device__ __forceinline__ void reg_op_k(cx<T> (&v)[N], cx<T> (&v2)[N], const OP &op, const Layout &l) {
    if constexpr ((1 << K) >= N) {
        return; // no such register bit at this register count
    }
    const u32 cm = op.rcmask, cv = op.rcval;
    const T ca = op.m[0].x, cb = op.m[0].y;
    const cx<T> m0 = op.m[0], m1 = op.m[1], m2 = op.m[2], m3 = op.m[3];
    auto pair = [&](cx<T> &x0, cx<T> &x1) {
        const cx<T> v0 = x0, v1 = x1;
        if constexpr (std::is_same_v<T, df> && MODE == RM_SROT_A) {
            const df nb = -cb;
            x0 = cx<T>{df_fma(v0.x, nb, v1.x), df_fma(v0.y, nb, v1.y)};
            x1 = cx<T>{df_fma(v1.x, cb, v0.x), df_fma(v1.y, cb, v0.y)};
        } else if constexpr (std::is_same_v<T, df> && MODE == RM_SROT_B) {
            x0 = cx<T>{df_fma(-v1.x, ca, v0.x), df_fma(-v1.y, ca, v0.y)};
            x1 = cx<T>{df_fma(v0.x, ca, v1.x), df_fma(v0.y, ca, v1.y)};
        } else if constexpr (MODE == RM_SROT_A) { // [[1, -b], [b, 1]]
            x0 = cx<T>{v0.x - cb * v1.x, v0.y - cb * v1.y};
            x1 = cx<T>{cb * v0.x + v1.x, cb * v0.y + v1.y};
        } else if constexpr (MODE == RM_SROT_B) { // [[a, -1], [1, a]]
            x0 = cx<T>{ca * v0.x - v1.x, ca * v0.y - v1.y};
            x1 = cx<T>{v0.x + ca * v1.x, v0.y + ca * v1.y};
        } else if constexpr (MODE == RM_SWAP) {
            x0 = v1;
            x1 = v0;
        } else { // general complex 2x2
            x0 = cfma(m1, v1, m0 * v0);
            x1 = cfma(m3, v1, m2 * v0);
        }
    };
#pragma unroll
    for (int i = 0; i < N; i++) {
        if (i & (1 << K)) {
            continue;
        }
        const int i1 = i | (1 << K);
        if constexpr (CTRL && MODE == RM_SWAP) {
            // controlled swap (CNOT, CSWAP): selects instead of a branch per pair
            const bool on = (l.at(i) & cm) == cv;
            auto cswap = [&](cx<T> &x0, cx<T> &x1) {
                const cx<T> v0 = x0, v1 = x1;
                x0 = on ? v1 : v0;
                x1 = on ? v0 : v1;
            };
            cswap(v[i], v[i1]);
            if constexpr (TWO) {
                cswap(v2[i], v2[i1]);
            }
            continue;
        }
        if (CTRL && ((l.at(i) & cm) != cv)) {
            continue;
        }
        pair(v[i], v[i1]);
        if constexpr (TWO) {
            pair(v2[i], v2[i1]);
        }
    }
}
template <int MODE, bool CTRL, bool TWO, class T, class OP, int N>
__device__ __forceinline__ void reg_op_m(cx<T> (&v)[N], cx<T> (&v2)[N], const OP &op, const Layout &l) {
    switch (op.rk) {
    case 0: reg_op_k<MODE, CTRL, T, 0, TWO>(v, v2, op, l); break;
    case 1: reg_op_k<MODE, CTRL, T, 1, TWO>(v, v2, op, l); break;
    case 2: reg_op_k<MODE, CTRL, T, 2, TWO>(v, v2, op, l); break;
    default: reg_op_k<MODE, CTRL, T, 3, TWO>(v, v2, op, l); break;
    }
}
template <bool TWO, class T, class OP, int N>
__device__ __forceinline__ void reg_op(cx<T> (&v)[N], cx<T> (&v2)[N], const OP &op, const Layout &l) {
    if (op.rcmask == 0) {
        switch (op.mode) {
        case RM_SROT_A: reg_op_m<RM_SROT_A, false, TWO>(v, v2, op, l); break;
        case RM_SROT_B: reg_op_m<RM_SROT_B, false, TWO>(v, v2, op, l); break;
        case RM_SWAP: reg_op_m<RM_SWAP, false, TWO>(v, v2, op, l); break;
        default: reg_op_m<RM_DENSE, false, TWO>(v, v2, op, l); break;
        }
    } else {
        switch (op.mode) {
        case RM_SROT_A: reg_op_m<RM_SROT_A, true, TWO>(v, v2, op, l); break;
        case RM_SROT_B: reg_op_m<RM_SROT_B, true, TWO>(v, v2, op, l); break;
        case RM_SWAP: reg_op_m<RM_SWAP, true, TWO>(v, v2, op, l); break;
        default: reg_op_m<RM_DENSE, true, TWO>(v, v2, op, l); break;
        }
    }
}

template <class T>
__device__ __forceinline__ cx<T> form_val(const DiagForm<T> &f, u64 gbase) {
    unsigned k = 0;
    for (int b = 0; b < f.nb; b++) {
        k = (k << 1) | static_cast<unsigned>((gbase >> f.bits[b]) & 1u);
    }
    return f.tab[k];
}


// Shared-memory state of the per-tile prologue (one slot per merged diagonal).
template <class T> struct TileShared {
    cx<T> scal[kMaxDiagOpsPerPass];
    u32 zl[kMaxDiagOpsPerPass];
    int ngen[kMaxDiagOpsPerPass];
    int gbit[kMaxDiagOpsPerPass][4];
    cx<T> gd0[kMaxDiagOpsPerPass][4];
    cx<T> gd1[kMaxDiagOpsPerPass][4];
    cx<T> factor;
};

// Apply pass `d` to tile g of register `a` (all threads of the CTA; the CTA
// has 2^(d.t - 4) threads and 2^d.t amplitudes of shared memory at `tile`).
// Op records of a pass, read by every register stage of every tile: either
// the global TileOp array or the fields register stages read (RegOpS),
// copied into shared memory once per CTA (STAGE).  Staging saves global
// loads per tile but costs registers: measured faster for the complex64
// kernels and the batched kernels; the single-register double-float kernel
// reads the global records (the staged form raised its spills six-fold at
// 128 registers).
template <class T, bool STAGE> using PassOpRec = std::conditional_t<STAGE, RegOpS<T>, TileOp<T>>;
template <class T, bool STAGE> constexpr size_t op_record_bytes(int nops) {
    return STAGE ? static_cast<size_t>(nops) * sizeof(RegOpS<T>) : 0;
}

// Stage the pass's op records (the fields register stages read) in shared
// memory; all threads of the CTA; the caller synchronises.
template <class T>
__device__ __forceinline__ void stage_ops(RegOpS<T> *sops, const TileOp<T> *__restrict__ ops, const TilePassDesc &d) {
    for (int k = threadIdx.x; k < d.nops; k += blockDim.x) {
        const TileOp<T> &o = ops[d.op_begin + k];
        RegOpS<T> r;
        r.kind = o.kind;
        r.mode = o.mode;
        r.rk = o.rk;
        r.diag_slot = o.diag_slot;
        r.rcmask = o.rcmask;
        r.rcval = o.rcval;
        r.has_table = o.has_table;
        r.table_off = o.table_off;
        r.gcmask = o.gcmask;
        r.gcval = o.gcval;
        r.ngforms = o.ngforms;
        r.gform_begin = o.gform_begin;
        r.nmforms = o.nmforms;
        r.mform_begin = o.mform_begin;
        for (int q = 0; q < 4; q++) {
            r.m[q] = o.m[q];
        }
        sops[k] = r;
    }
}

// The records of pass d for tile_reg_run, indexed from d.op_begin: staged at
// smem_after_tile (all threads; the caller synchronises) or in place.
template <class T, bool STAGE>
__device__ __forceinline__ const PassOpRec<T, STAGE> *op_records(unsigned char *smem_after_tile, const TileOp<T> *ops,
                                                             const TilePassDesc &d) {
    if constexpr (STAGE) {
        RegOpS<T> *sops = reinterpret_cast<RegOpS<T> *>(smem_after_tile);
        stage_ops(sops, ops, d);
        return sops;
    } else {
        return ops + d.op_begin;
    }
}

// Adjoint reduction in a register stage (two-register kernel): this
// thread's share of  sum_j [(j & P) == pv] Re or Im( conj(b_j) a_k ) with
// k = j ^ flip, signed by the parity of (k & yz) and of the tile's global
// Y|Z bits.  XR = the flip as a register-slot mask (compile time, so both
// slots stay in registers).  Products and the running sum in double-float
// (complex64 / double-float registers) or FP64 (complex128 in FP64).
template <class T, int XR, bool RE, int N>
__device__ __forceinline__ double reduce_slots(const cx<T> (&a)[N], const cx<T> (&b)[N], const Layout &l,
                                               u32 pm, u32 pv, u32 yz, unsigned gpar) {
    if constexpr (XR >= N) {
        return 0.0; // no such register bit at this register count
    }
    if constexpr (std::is_same_v<T, double>) {
        double acc = 0.0;
#pragma unroll
        for (int i = 0; i < N; i++) {
            const cx<double> p = b[i], q = a[i ^ XR];
            // Re: px qx + py qy;  Im: px qy - py qx
            double z = RE ? fma(p.y, q.y, p.x * q.x) : fma(-p.y, q.x, p.x * q.y);
            z = sflip(z, (static_cast<unsigned>(__popc(l.at(i ^ XR) & yz)) ^ gpar) & 1u);
            acc += ((l.at(i) & pm) == pv) ? z : 0.0;
        }
        return acc;
    } else {
        df acc{0.f, 0.f};
#pragma unroll
        for (int i = 0; i < N; i++) {
            df px, py, qx, qy;
            if constexpr (std::is_same_v<T, df>) {
                px = b[i].x, py = b[i].y, qx = a[i ^ XR].x, qy = a[i ^ XR].y;
            } else {
                px = df(b[i].x), py = df(b[i].y), qx = df(a[i ^ XR].x), qy = df(a[i ^ XR].y);
            }
            // Re: px qx + py qy;  Im: px qy - py qx
            df z = RE ? df_fma(px * qx, py, qy) : df_fma(px * qy, -py, qx);
            z = sflip(z, (static_cast<unsigned>(__popc(l.at(i ^ XR) & yz)) ^ gpar) & 1u);
            if ((l.at(i) & pm) != pv) { // outside the projector: adds zero
                z = df{0.f, 0.f};
            }
            acc = acc + z;
        }
        return df_to_double(acc);
    }
}

// Apply pass d to tile g.  DUAL (adjoint sweep): the same ops to a second
// register b (its tile at tileb), and the pass's reductions (TK_REDUCE, in
// register stages) accumulated per warp into s_part[slot * nwarps + warp];
// s_f2[k] = |product of the first k merged diagonals' tile scalars|^2, the
// deferred factor a reduction after k of them must include.
template <class T, class SI = T, class SO = T, bool DUAL = false, int RBT = kRegBits, class REC>
__device__ __forceinline__ void tile_reg_run(const cx<SI> *ain, cx<SO> *aout, const TilePassDesc &d,
                                             const TileOp<T> *__restrict__ ops, const DiagForm<T> *__restrict__ forms,
                                             const cx<T> *__restrict__ tables, const StageDesc *__restrict__ stages,
                                             u64 g, cx<T> *tile, TileShared<T> &sh, const REC *recs,
                                             const cx<SI> *bin = nullptr, cx<SO> *bout = nullptr,
                                             cx<T> *tileb = nullptr, double *s_part = nullptr,
                                             double *s_f2 = nullptr) {
    constexpr int NRT = 1 << RBT; // amplitudes per thread and register
    const int w = d.t - RBT;
    const u32 tid = threadIdx.x;
    const int lane = static_cast<int>(tid & 31u);
    const int warp = static_cast<int>(tid >> 5);
    const int nwarps = static_cast<int>(blockDim.x >> 5);
    cx<T> v[NRT];
    cx<T> vb[DUAL ? NRT : 1];
    // global offset of canonical slot i of this thread: the local->global map
    // is a bit deposit, so it splits into a thread part and a slot part
    const u64 off_t = local_offset_r(tid, d);
    // canonical slot bits are local bits w..w+3 = global bits hb[w-L .. w-L+3]
    const int g0 = d.hb[w - d.L], g1 = d.hb[w - d.L + 1], g2 = d.hb[w - d.L + 2];
    const int g3 = RBT > 3 ? d.hb[w - d.L + 3] : 0;
    auto off_r = [&](int i) -> u64 {
        return ((i & 1) ? (u64{1} << g0) : 0) | ((i & 2) ? (u64{1} << g1) : 0) | ((i & 4) ? (u64{1} << g2) : 0) |
               ((i & 8) ? (u64{1} << g3) : 0);
    };
    const Layout canon = canonical_layout(tid, w);

    u64 gbase = g << d.L;
    for (int m = 0; m < d.H; m++) {
        const int p = d.hb[m];
        gbase = ((gbase >> p) << (p + 1)) | (gbase & ((u64{1} << p) - 1));
    }
    const u64 tbase = gbase | off_t;
#pragma unroll
    for (int i = 0; i < NRT; i++) {
        v[i] = ld_conv<T, SI>(ld_stream(&ain[tbase | off_r(i)]));
    }
    if constexpr (DUAL) {
#pragma unroll
        for (int i = 0; i < NRT; i++) {
            vb[i] = ld_conv<T, SI>(ld_stream(&bin[tbase | off_r(i)]));
        }
    }
    // prologue: tile-uniform parts of every merged diagonal, one warp per op
    int slot = 0;
    for (int oi = 0; oi < d.nops; oi++) {
        const REC &op = recs[oi];
        if (op.kind != TK_DIAGTAB) {
            continue;
        }
        if ((slot % nwarps) == warp) {
            cx<T> sc{1, 0};
            if ((gbase & op.gcmask) == op.gcval) {
                for (int f = lane; f < op.ngforms; f += 32) {
                    sc = sc * form_val(forms[op.gform_begin + f], gbase);
                }
            }
            u32 zl = 0;
            bool gen = false;
            cx<T> d0{1, 0}, d1{1, 0};
            int lb = 0;
            if (lane < op.nmforms && (gbase & op.gcmask) == op.gcval) {
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
            for (int mm = 16; mm > 0; mm >>= 1) {
                sc = sc * shx(sc, mm);
                zl ^= __shfl_xor_sync(0xffffffffu, zl, mm);
            }
            const unsigned gm = __ballot_sync(0xffffffffu, gen);
            if (gen) {
                const int k = __popc(gm & ((1u << lane) - 1u));
                if (k < 4) {
                    sh.gbit[slot][k] = lb;
                    sh.gd0[slot][k] = d0;
                    sh.gd1[slot][k] = d1;
                }
            }
            if (lane == 0) {
                sh.scal[slot] = sc;
                sh.zl[slot] = zl;
                sh.ngen[slot] = min(__popc(gm), 4);
            }
        }
        slot++;
    }
    __syncthreads();
    if (tid == 0) {
        cx<T> f{from_double<T>(d.pass_scale), from_double<T>(0.0)};
        for (int s = 0; s < d.ndiag; s++) {
            f = f * sh.scal[s];
        }
        sh.factor = f;
        if constexpr (DUAL) {
            double f2 = 1.0;
            s_f2[0] = f2;
            for (int s = 0; s < d.ndiag; s++) {
                const double x = static_cast<double>(sh.scal[s].x), y = static_cast<double>(sh.scal[s].y);
                f2 *= x * x + y * y;
                s_f2[s + 1] = f2;
            }
        }
    }

    Layout cur = canon;
    bool cur_canon = true;
    int cur_stage = -1;
    for (int si = 0; si < d.nstages; si++) {
        const StageDesc *st = &stages[d.stage_begin + si];
        if (st->kind == 0) {
            if (cur_stage != si) {
                const Layout nl = stage_layout(st, tid, w);
                to_smem(tile, v, cur);
                if constexpr (DUAL) {
                    to_smem(tileb, vb, cur);
                }
                __syncthreads();
                from_smem(tile, v, nl);
                if constexpr (DUAL) {
                    from_smem(tileb, vb, nl);
                }
                __syncthreads();
                cur = nl;
                cur_canon = false;
                cur_stage = si;
            }
            for (int oi = st->op_begin; oi < st->op_begin + st->nops; oi++) {
                const REC &op = recs[oi - d.op_begin];
                if ((gbase & op.gcmask) != op.gcval) {
                    continue;
                }
                if (op.kind == TK_DIAGTAB) {
                    const int s = op.diag_slot;
                    const u32 zl = sh.zl[s];
                    const int ngen = sh.ngen[s];
                    const cx<T> *tab = tables + op.table_off;
                    if (op.has_table && zl == 0) {
#pragma unroll
                        for (int i = 0; i < NRT; i++) {
                            const cx<T> tv = tab[cur.at(i)];
                            v[i] = tv * v[i];
                            if constexpr (DUAL) {
                                vb[i] = tv * vb[i];
                            }
                        }
                    } else if (op.has_table) {
#pragma unroll
                        for (int i = 0; i < NRT; i++) {
                            const u32 j = cur.at(i);
                            const cx<T> tv = tab[j];
                            const unsigned fl = static_cast<unsigned>(__popc(j & zl) & 1);
                            v[i] = cflip(tv * v[i], fl);
                            if constexpr (DUAL) {
                                vb[i] = cflip(tv * vb[i], fl);
                            }
                        }
                    } else if (zl) {
#pragma unroll
                        for (int i = 0; i < NRT; i++) {
                            const unsigned fl = static_cast<unsigned>(__popc(cur.at(i) & zl) & 1);
                            v[i] = cflip(v[i], fl);
                            if constexpr (DUAL) {
                                vb[i] = cflip(vb[i], fl);
                            }
                        }
                    }
                    for (int f = 0; f < ngen; f++) {
                        const int gb = sh.gbit[s][f];
                        const cx<T> g0 = sh.gd0[s][f], g1 = sh.gd1[s][f];
#pragma unroll
                        for (int i = 0; i < NRT; i++) {
                            const cx<T> gv = ((cur.at(i) >> gb) & 1u) ? g1 : g0;
                            v[i] = gv * v[i];
                            if constexpr (DUAL) {
                                vb[i] = gv * vb[i];
                            }
                        }
                    }
                } else if (op.kind == TK_PARITY) {
                    const TileOp<T> &po = ops[oi];
#pragma unroll
                    for (int i = 0; i < NRT; i++) {
                        const u64 idx = gbase | local_offset_r(cur.at(i), d);
                        if ((idx & po.cmask) != po.cval) {
                            if (po.zero_outside) {
                                v[i] = cx<T>{0, 0};
                                if constexpr (DUAL) {
                                    vb[i] = cx<T>{0, 0};
                                }
                            }
                            continue;
                        }
                        const cx<T> pv = (__popcll(idx & po.pmask) & 1) ? op.m[1] : op.m[0];
                        v[i] = pv * v[i];
                        if constexpr (DUAL) {
                            vb[i] = pv * vb[i];
                        }
                    }
                } else if (DUAL && op.kind == TK_REDUCE) {
                    if constexpr (DUAL) {
                        const TileOp<T> &ro = ops[oi];
                        const unsigned gpar = static_cast<unsigned>(__popcll(gbase & ro.pmask) & 1);
                        const bool want_re = (ro.mode & 1) != 0;
                        double z;
                        // the flip slot mask and Re / Im as compile-time cases
                        // (the register count of the adjoint kernel: XR <= 4)
                        const u32 pm = ro.rcmask, pv = ro.lcval, yz = ro.lo0;
                        switch (ro.tcmask * 2 + (want_re ? 1 : 0)) {
                        case 0: z = reduce_slots<T, 0, false>(v, vb, cur, pm, pv, yz, gpar); break;
                        case 1: z = reduce_slots<T, 0, true>(v, vb, cur, pm, pv, yz, gpar); break;
                        case 2: z = reduce_slots<T, 1, false>(v, vb, cur, pm, pv, yz, gpar); break;
                        case 3: z = reduce_slots<T, 1, true>(v, vb, cur, pm, pv, yz, gpar); break;
                        case 4: z = reduce_slots<T, 2, false>(v, vb, cur, pm, pv, yz, gpar); break;
                        case 5: z = reduce_slots<T, 2, true>(v, vb, cur, pm, pv, yz, gpar); break;
                        case 8: z = reduce_slots<T, 4, false>(v, vb, cur, pm, pv, yz, gpar); break;
                        case 9: z = reduce_slots<T, 4, true>(v, vb, cur, pm, pv, yz, gpar); break;
                        case 16: z = reduce_slots<T, 8, false>(v, vb, cur, pm, pv, yz, gpar); break;
                        default: z = reduce_slots<T, 8, true>(v, vb, cur, pm, pv, yz, gpar); break;
                        }
                        if (ro.mode & 2) {
                            z = -z;
                        }
#pragma unroll
                        for (int m = 16; m > 0; m >>= 1) {
                            z += __shfl_xor_sync(0xffffffffu, z, m);
                        }
                        if (lane == 0) {
                            s_part[ro.diag_slot * nwarps + warp] += z * ro.rmul * s_f2[ro.tcval];
                        }
                    }
                } else if constexpr (DUAL) {
                    reg_op<true>(v, vb, op, cur);
                } else {
                    reg_op<false>(v, v, op, cur);
                }
            }
        } else {
            // shared-memory stage: two-target ops on the staged tile(s)
            to_smem(tile, v, cur);
            if constexpr (DUAL) {
                to_smem(tileb, vb, cur);
            }
            __syncthreads();
            const u32 T_ = 1u << d.t;
            auto smem_op = [&](cx<T> *tl, const TileOp<T> &op) {
                if (op.kind == TK_DENSE2) {
                    const u32 nq = T_ >> op.nlins;
                    for (u32 p = tid; p < nq; p += blockDim.x) {
                        const u32 j0 = insert_zeros_r(p, op.lins, op.nlins) | op.lcval;
                        const u32 ix[4] = {swz<T>(j0), swz<T>(j0 | op.lo1), swz<T>(j0 | op.lo0),
                                           swz<T>(j0 | op.lo0 | op.lo1)};
                        cx<T> x[4];
#pragma unroll
                        for (int r = 0; r < 4; r++) {
                            x[r] = tl[ix[r]];
                        }
#pragma unroll
                        for (int r = 0; r < 4; r++) {
                            cx<T> acc = op.m[4 * r] * x[0];
                            acc = cfma(op.m[4 * r + 1], x[1], acc);
                            acc = cfma(op.m[4 * r + 2], x[2], acc);
                            acc = cfma(op.m[4 * r + 3], x[3], acc);
                            tl[ix[r]] = acc;
                        }
                    }
                } else { // two-amplitude op with general offsets
                    const u32 np = T_ >> op.nlins;
                    for (u32 p = tid; p < np; p += blockDim.x) {
                        const u32 j0 = insert_zeros_r(p, op.lins, op.nlins) | op.lcval;
                        cx<T> &x0 = tl[swz<T>(j0 | op.lo0)];
                        cx<T> &x1 = tl[swz<T>(j0 | op.lo1)];
                        const cx<T> v0 = x0, v1 = x1;
                        if (op.mode == RM_SWAP) {
                            x0 = v1;
                            x1 = v0;
                        } else {
                            x0 = cfma(op.m[1], v1, op.m[0] * v0);
                            x1 = cfma(op.m[3], v1, op.m[2] * v0);
                        }
                    }
                }
            };
            for (int oi = st->op_begin; oi < st->op_begin + st->nops; oi++) {
                const TileOp<T> &op = ops[oi];
                if ((gbase & op.gcmask) == op.gcval) {
                    smem_op(tile, op);
                    if constexpr (DUAL) {
                        smem_op(tileb, op);
                    }
                }
                __syncthreads();
            }
            from_smem(tile, v, canon);
            if constexpr (DUAL) {
                from_smem(tileb, vb, canon);
            }
            __syncthreads();
            cur = canon;
            cur_canon = true;
            cur_stage = -1;
        }
    }
    if (!cur_canon) {
        to_smem(tile, v, cur);
        if constexpr (DUAL) {
            to_smem(tileb, vb, cur);
        }
        __syncthreads();
        from_smem(tile, v, canon);
        if constexpr (DUAL) {
            from_smem(tileb, vb, canon);
        }
    }
    __syncthreads();
    const cx<T> f = sh.factor;
#pragma unroll
    for (int i = 0; i < NRT; i++) {
        st_stream(&aout[tbase | off_r(i)], st_conv<SO, T>(f * v[i]));
    }
    if constexpr (DUAL) {
#pragma unroll
        for (int i = 0; i < NRT; i++) {
            st_stream(&bout[tbase | off_r(i)], st_conv<SO, T>(f * vb[i]));
        }
    }
    __syncthreads();
}

} // namespace

} // namespace plgb
