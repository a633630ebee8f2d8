// Measurement and linear-algebra kernels (sm_103a).  All reductions are
// warp-shuffle + shared-memory tree reductions into per-block partials,
// followed by a fixed-order final sum, so a result does not depend on
// scheduling.  Accumulation is in double for both precisions, except the
// Pauli-sum kernels, which multiply and add in double-float arithmetic (the
// FP32 pipe; FP64 runs at 1/64 of its rate on GB300) and convert once.
//
// Reference semantics: pennylane_lightning/core/simulators/lightning_qubit/
// measurements/MeasurementsLQubit.hpp (probs :90-163, expval :213-394),
// ExpValFunc.hpp (:69-335), utils/LinearAlgebra.hpp innerProdC (:122-145),
// observables/ObservablesLQubit.hpp HamiltonianApplyInPlace (:156-251).
#include "df.cuh"
#include "kernels.hpp"

#include <type_traits>

namespace plgb {

template <int NOUT, int THREADS = kReduceThreads>
__device__ __forceinline__ void block_reduce_store(double (&v)[NOUT], double *partials) {
    static_assert(THREADS % 32 == 0 && THREADS <= 1024, "whole warps, at most 32");
    __shared__ double sh[NOUT][THREADS / 32];
#pragma unroll
    for (int o = 0; o < NOUT; o++) {
        double x = v[o];
#pragma unroll
        for (int d = 16; d > 0; d >>= 1) {
            x += __shfl_down_sync(0xffffffffu, x, d);
        }
        if ((threadIdx.x & 31) == 0) {
            sh[o][threadIdx.x >> 5] = x;
        }
    }
    __syncthreads();
    if (threadIdx.x < 32) {
#pragma unroll
        for (int o = 0; o < NOUT; o++) {
            double x = threadIdx.x < (THREADS / 32) ? sh[o][threadIdx.x] : 0.0;
#pragma unroll
            for (int d = 16; d > 0; d >>= 1) {
                x += __shfl_down_sync(0xffffffffu, x, d);
            }
            if (threadIdx.x == 0) {
                partials[static_cast<size_t>(blockIdx.x) * NOUT + o] = x;
            }
        }
    }
}

template <int NOUT> __global__ void k_finalize(const double *__restrict__ partials, int nblocks, double *out) {
    // one warp per output, fixed order
    const int o = threadIdx.x >> 5;
    const int lane = threadIdx.x & 31;
    if (o >= NOUT) {
        return;
    }
    double x = 0.0;
    for (int b = lane; b < nblocks; b += 32) {
        x += partials[static_cast<size_t>(b) * NOUT + o];
    }
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) {
        x += __shfl_down_sync(0xffffffffu, x, d);
    }
    if (lane == 0) {
        out[o] = x;
    }
}

template <int NOUT> static void finalize(cudaStream_t s, const double *partials, int nblocks, double *out) {
    k_finalize<NOUT><<<1, 32 * NOUT, 0, s>>>(partials, nblocks, out);
    cuda_check(cudaGetLastError(), "k_finalize launch");
    note_launch();
}

static int reduce_grid(u64 work) {
    const u64 want = (work + kReduceThreads - 1) / kReduceThreads;
    return static_cast<int>(want < static_cast<u64>(kReduceBlocks) ? (want < 1 ? 1 : want) : kReduceBlocks);
}

#define GRID_STRIDE(i, N)                                                                                         \
    for (u64 i = static_cast<u64>(blockIdx.x) * blockDim.x + threadIdx.x; i < (N);                             \
         i += static_cast<u64>(gridDim.x) * blockDim.x)

// ---------------------------------------------------------------------------
template <class T> __global__ void __launch_bounds__(kReduceThreads) k_norm2(const cx<T> *__restrict__ a, u64 N, double *partials) {
    double v[1] = {0.0};
    GRID_STRIDE(i, N) {
        const cx<T> x = a[i];
        v[0] += static_cast<double>(x.x) * x.x + static_cast<double>(x.y) * x.y;
    }
    block_reduce_store<1>(v, partials);
}
template <class T> void reduce_norm2(cudaStream_t s, const cx<T> *sv, u64 N, double *partials, double *out) {
    const int g = reduce_grid(N);
    k_norm2<T><<<g, kReduceThreads, 0, s>>>(sv, N, partials);
    cuda_check(cudaGetLastError(), "k_norm2 launch");
    note_launch();
    finalize<1>(s, partials, g, out);
}

// <a|b> = sum conj(a_i) b_i
template <class T>
__global__ void __launch_bounds__(kReduceThreads) k_inner(const cx<T> *__restrict__ a, const cx<T> *__restrict__ b, u64 N, double *partials) {
    double v[2] = {0.0, 0.0};
    GRID_STRIDE(i, N) {
        const cx<T> x = a[i];
        const cx<T> y = b[i];
        v[0] += static_cast<double>(x.x) * y.x + static_cast<double>(x.y) * y.y;
        v[1] += static_cast<double>(x.x) * y.y - static_cast<double>(x.y) * y.x;
    }
    block_reduce_store<2>(v, partials);
}
template <class T>
void reduce_inner(cudaStream_t s, const cx<T> *a, const cx<T> *b, u64 N, double *partials, double *out) {
    const int g = reduce_grid(N);
    k_inner<T><<<g, kReduceThreads, 0, s>>>(a, b, N, partials);
    cuda_check(cudaGetLastError(), "k_inner launch");
    note_launch();
    finalize<2>(s, partials, g, out);
}

// Named one-wire observables (ExpValFunc.hpp:69-90 with the per-name cores of
// MeasurementsLQubit.hpp:247-305).
template <class T, int KIND>
__global__ void __launch_bounds__(kReduceThreads) k_expval1(const cx<T> *__restrict__ a, u64 half, int tbit, double *partials) {
    double v[1] = {0.0};
    const u64 tm = u64{1} << tbit;
    GRID_STRIDE(k, half) {
        const u64 i0 = insert_zero(k, tbit);
        const cx<T> p = a[i0];
        const cx<T> q = a[i0 | tm];
        const double px = p.x, py = p.y, qx = q.x, qy = q.y;
        if constexpr (KIND == 0) {
            v[0] += 2.0 * (px * qx + py * qy);
        } else if constexpr (KIND == 1) {
            v[0] += 2.0 * (px * qy - py * qx);
        } else if constexpr (KIND == 2) {
            v[0] += (px * px + py * py) - (qx * qx + qy * qy);
        } else {
            v[0] += 0.70710678118654752440 * ((px * px + py * py) - (qx * qx + qy * qy) + 2.0 * (px * qx + py * qy));
        }
    }
    block_reduce_store<1>(v, partials);
}
template <class T>
void reduce_expval1(cudaStream_t s, const cx<T> *sv, u64 N, int tbit, int kind, double *partials, double *out) {
    const u64 half = N >> 1;
    const int g = reduce_grid(half);
    switch (kind) {
    case 0: k_expval1<T, 0><<<g, kReduceThreads, 0, s>>>(sv, half, tbit, partials); break;
    case 1: k_expval1<T, 1><<<g, kReduceThreads, 0, s>>>(sv, half, tbit, partials); break;
    case 2: k_expval1<T, 2><<<g, kReduceThreads, 0, s>>>(sv, half, tbit, partials); break;
    default: k_expval1<T, 3><<<g, kReduceThreads, 0, s>>>(sv, half, tbit, partials); break;
    }
    cuda_check(cudaGetLastError(), "k_expval1 launch");
    note_launch();
    finalize<1>(s, partials, g, out);
}

// ---------------------------------------------------------------------------
// Pauli words.  With P|k> = i^ny (-1)^{|k & yz|} |k ^ x>, the expectation
// over a pair (j, j' = j ^ x) is  sum_t c_t Re( i^ny [ s(j') A + s(j) conj(A) ] )
// with A = conj(psi_j) psi_j' and s(k) = (-1)^{|k & yz|}.  One read of the
// state serves every term of a flip-mask group.
// ---------------------------------------------------------------------------
__device__ __forceinline__ double term_pair(const PauliTerm &t, u64 j, u64 jp, double ar, double ai) {
    const double s = (__popcll(j & t.yz) & 1) ? -1.0 : 1.0;
    const double sp = (__popcll(jp & t.yz) & 1) ? -1.0 : 1.0;
    // i^ny * ((s'+s) ar + i (s'-s) ai), real part
    switch (t.ny4) {
    case 0: return (sp + s) * ar;
    case 1: return -(sp - s) * ai;
    case 2: return -(sp + s) * ar;
    default: return (sp - s) * ai;
    }
}

template <class T> __device__ __forceinline__ df to_df(T x) {
    if constexpr (std::is_same_v<T, double>) {
        return df_from_bits(x);
    } else {
        return df{x, 0.f};
    }
}
template <class T> __device__ __forceinline__ T from_df(df x) {
    if constexpr (std::is_same_v<T, double>) {
        return df_to_double(x);
    } else {
        return __fadd_rn(x.hi, x.lo);
    }
}
// <psi| sum_t c_t P_t |psi> for one flip-mask group.  Products and sums in
// double-float arithmetic (FP32 pipe; complex128 amplitudes split with
// integer operations), one conversion per thread before the block reduction.
template <class T>
__global__ void __launch_bounds__(kReduceThreads) k_pauli_group(const cx<T> *__restrict__ a, u64 N, const __grid_constant__ PauliGroup g,
                                                               double *partials) {
    __shared__ df sc[kMaxTermsPerGroup];
    for (int t = static_cast<int>(threadIdx.x); t < g.nterms; t += static_cast<int>(blockDim.x)) {
        sc[t] = df(g.t[t].coeff);
    }
    __syncthreads();
    df acc{0.f, 0.f};
    if (g.x == 0) {
        GRID_STRIDE(j, N) {
            const cx<T> p = a[j];
            const df pr = to_df<T>(p.x), pi = to_df<T>(p.y);
            const df w = df_fma(pr * pr, pi, pi);
            df f{0.f, 0.f};
            for (int t = 0; t < g.nterms; t++) {
                f = (__popcll(j & g.t[t].yz) & 1) ? f - sc[t] : f + sc[t];
            }
            acc = df_fma(acc, w, f);
        }
    } else {
        const u64 half = N >> 1;
        GRID_STRIDE(k, half) {
            const u64 j = insert_zero(k, g.hb);
            const u64 jp = j ^ g.x;
            const cx<T> p = a[j];
            const cx<T> q = a[jp];
            const df pr = to_df<T>(p.x), pi = to_df<T>(p.y), qr = to_df<T>(q.x), qi = to_df<T>(q.y);
            // conj(p) q = ar + i ai
            const df ar = df_fma(pr * qr, pi, qi);
            const df ai = df_fma(pr * qi, -pi, qr);
            // per term (term_pair): i^ny ((s' + s) ar + i (s' - s) ai), real part;
            // s' + s and s' - s are 0 or +-2
            df A{0.f, 0.f}, B{0.f, 0.f};
            for (int t = 0; t < g.nterms; t++) {
                const bool s = (__popcll(j & g.t[t].yz) & 1) != 0, sp = (__popcll(jp & g.t[t].yz) & 1) != 0;
                const df c2 = sc[t] + sc[t];
                switch (g.t[t].ny4) {
                case 0: if (s == sp) { A = s ? A - c2 : A + c2; } break;
                case 1: if (s != sp) { B = sp ? B + c2 : B - c2; } break;
                case 2: if (s == sp) { A = s ? A + c2 : A - c2; } break;
                default: if (s != sp) { B = sp ? B - c2 : B + c2; } break;
                }
            }
            acc = df_fma(df_fma(acc, A, ar), B, ai);
        }
    }
    double v[1] = {df_to_double(acc)};
    block_reduce_store<1>(v, partials);
}
template <class T>
void reduce_pauli_group(cudaStream_t s, const cx<T> *sv, u64 N, const PauliGroup &g, double *partials, double *out) {
    const int grid = reduce_grid(g.x == 0 ? N : N >> 1);
    k_pauli_group<T><<<grid, kReduceThreads, 0, s>>>(sv, N, g, partials);
    cuda_check(cudaGetLastError(), "k_pauli_group launch");
    note_launch();
    finalize<1>(s, partials, grid, out);
}

// Pauli words by passes (kernels.hpp, PauliPass): the tile is staged in
// shared memory as double-float pairs (each amplitude converted once), then
// every word of the pass is evaluated from it.  Products and sums in
// double-float arithmetic on the FP32 pipe.
constexpr int kPassThreads = 256;
template <class T>
__global__ void __launch_bounds__(kPassThreads) k_pauli_pass(const cx<T> *__restrict__ a, const __grid_constant__ PauliPass d,
                                                             double *partials) {
    extern __shared__ float4 tl[]; // local amplitude jj: (re.hi, re.lo, im.hi, im.lo)
    const unsigned tid = threadIdx.x;
    const unsigned T_ = 1u << d.t;
    // global offset of local index jj = r * 256 + tid: a thread part and a
    // part per r (local bits 0-7 from tid, the rest from r)
    u64 off_t = 0;
    for (int q = 0; q < 8 && q < d.t; q++) {
        off_t |= static_cast<u64>((tid >> q) & 1u) << d.lbit[q];
    }
    df acc[kPassTerms];
#pragma unroll
    for (int w = 0; w < kPassTerms; w++) {
        acc[w] = df{0.f, 0.f};
    }
    for (u64 tile = blockIdx.x; tile < d.ntiles; tile += gridDim.x) {
        u64 base = 0;
        {
            u64 tt = tile;
            for (int q = 0; q < d.nglob; q++) {
                base |= (tt & 1u) << d.glob[q];
                tt >>= 1;
            }
        }
        for (unsigned r = 0; r * kPassThreads < T_; r++) {
            const unsigned jj = r * kPassThreads + tid;
            if (jj >= T_) {
                break;
            }
            u64 off = base | off_t;
            for (int q = 8; q < d.t; q++) {
                off |= static_cast<u64>((r >> (q - 8)) & 1u) << d.lbit[q];
            }
            const cx<T> v = a[off];
            const df re = to_df<T>(v.x), im = to_df<T>(v.y);
            tl[jj] = make_float4(re.hi, re.lo, im.hi, im.lo);
        }
        __syncthreads();
#pragma unroll
        for (int w = 0; w < kPassTerms; w++) {
            if (w >= d.nterms) {
                break;
            }
            const PauliPassTerm &pt = d.term[w];
            const unsigned tpar = static_cast<unsigned>(__popcll(base & pt.yz)) & 1u;
            if (pt.x == 0) {
                for (unsigned j = tid; j < T_; j += kPassThreads) {
                    const float4 p = tl[j];
                    const df pr{p.x, p.y}, pi{p.z, p.w};
                    const df v = df_fma(pr * pr, pi, pi);
                    const bool neg = ((static_cast<unsigned>(__popc(j & pt.yzl)) ^ tpar) & 1u) != 0;
                    acc[w] = neg ? acc[w] - v : acc[w] + v;
                }
            } else {
                const unsigned lo = (1u << pt.hb) - 1u;
                for (unsigned k = tid; k < (T_ >> 1); k += kPassThreads) {
                    const unsigned j = ((k >> pt.hb) << (pt.hb + 1)) | (k & lo);
                    const float4 p = tl[j], q = tl[j ^ pt.x];
                    const df pr{p.x, p.y}, pi{p.z, p.w}, qr{q.x, q.y}, qi{q.z, q.w};
                    // conj(p) q = (pr qr + pi qi) + i (pr qi - pi qr)
                    const df v = pt.im ? df_fma(pr * qi, -pi, qr) : df_fma(pr * qr, pi, qi);
                    const bool neg = ((static_cast<unsigned>(__popc(j & pt.yzl)) ^ tpar) & 1u) != 0;
                    acc[w] = neg ? acc[w] - v : acc[w] + v;
                }
            }
        }
        __syncthreads();
    }
    double v[kPassTerms];
#pragma unroll
    for (int w = 0; w < kPassTerms; w++) {
        v[w] = df_to_double(acc[w]);
    }
    block_reduce_store<kPassTerms>(v, partials);
}
// Tiles of 2^12 amplitudes (registers of 12 or more qubits): the same sums
// with less index and sign work per pair, and the loads of the next tile in
// flight while the current one is evaluated.  One 512-thread CTA per SM;
// tiles arrive by 16-byte (complex64: 8-byte) asynchronous copies into two
// raw buffers; a complex128 tile is converted in place to double-float
// pairs (16 bytes either way) by the thread that copied each amplitude.
// Thread tid takes pairs k = r * 512 + tid (r < 4) of a non-diagonal word;
// j (k with a zero at the word's top flip bit) is a thread part computed
// once per word and tile OR the host's part jr[r], and the sign
// (-1)^{|j & yz|} splits the same way (thread part, tile part from the
// global bits, srm bit r).  A pair's value keeps the products' rounding
// errors (TwoProd by FMA, TwoSum); each word's sum is a float pair (A, L):
// A accumulates by TwoSum, L collects the low parts.  The pairs of the 16
// words live in shared memory behind the buffers (one float2 per word and
// thread), read and written once per word and tile.
struct PassAcc {
    float a, l;
};
// s + c = (ah + al)(bh + bl) + (ch + cl)(dh + dl), without the lo x lo terms
__device__ __forceinline__ void pass_dot2(float ah, float al, float bh, float bl, float ch, float cl, float dh,
                                          float dl, float &s, float &c) {
    const float h1 = __fmul_rn(ah, bh);
    const float e1 = __fmaf_rn(ah, bh, -h1);
    const float h2 = __fmul_rn(ch, dh);
    const float e2 = __fmaf_rn(ch, dh, -h2);
    s = __fadd_rn(h1, h2);
    const float bb = __fsub_rn(s, h1);
    const float es = __fadd_rn(__fsub_rn(h1, __fsub_rn(s, bb)), __fsub_rn(h2, bb));
    float t = __fmaf_rn(ah, bl, e1);
    t = __fmaf_rn(al, bh, t);
    t = __fmaf_rn(ch, dl, t);
    t = __fmaf_rn(cl, dh, t);
    c = __fadd_rn(t, __fadd_rn(e2, es));
}
// s + c = a b + c d for floats (exact)
__device__ __forceinline__ void pass_dot2f(float a, float b, float c_, float d, float &s, float &c) {
    const float h1 = __fmul_rn(a, b);
    const float e1 = __fmaf_rn(a, b, -h1);
    const float h2 = __fmul_rn(c_, d);
    const float e2 = __fmaf_rn(c_, d, -h2);
    s = __fadd_rn(h1, h2);
    const float bb = __fsub_rn(s, h1);
    const float es = __fadd_rn(__fsub_rn(h1, __fsub_rn(s, bb)), __fsub_rn(h2, bb));
    c = __fadd_rn(e1, __fadd_rn(e2, es));
}
// acc += sg * (s + c), sg = +-1 (sg * s is exact)
__device__ __forceinline__ void pass_accumulate(PassAcc &acc, float sg, float s, float c) {
    const float b = __fmul_rn(sg, s);
    const float a1 = __fadd_rn(acc.a, b);
    const float bb = __fsub_rn(a1, acc.a);
    const float ea = __fadd_rn(__fsub_rn(acc.a, __fsub_rn(a1, bb)), __fsub_rn(b, bb));
    acc.l = __fadd_rn(acc.l, __fmaf_rn(sg, c, ea));
    acc.a = a1;
}
__device__ __forceinline__ float pass_sign(unsigned bit) { return bit ? -1.f : 1.f; }

__device__ __forceinline__ void pass_cp_async(unsigned dst, const void *src, int bytes) {
    if (bytes == 16) {
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(dst), "l"(src) : "memory");
    } else {
        asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(dst), "l"(src) : "memory");
    }
}

constexpr int kPass12Threads = 512;
template <class T> constexpr size_t pass12_smem() {
    return 2 * (sizeof(cx<T>) << 12) + sizeof(float2) * kPassTerms * kPass12Threads;
}
template <class T>
__global__ void __launch_bounds__(kPass12Threads, 1)
    k_pauli_pass12(const cx<T> *__restrict__ a, const __grid_constant__ PauliPass d, double *partials) {
    extern __shared__ __align__(16) unsigned char smem[];
    constexpr bool kDF = sizeof(T) == 8; // complex128: double-float pairs
    constexpr unsigned kT = 1u << 12;
    constexpr unsigned kAmp = sizeof(cx<T>);
    constexpr unsigned kTileBytes = kAmp * kT;
    constexpr int kRows = kT / kPass12Threads; // amplitudes per thread and tile (8)
    float2 *sums = reinterpret_cast<float2 *>(smem + 2 * kTileBytes); // [word][thread]
    const unsigned tid = threadIdx.x;
    const unsigned s0 = static_cast<unsigned>(__cvta_generic_to_shared(smem));
    u64 off_t = 0;
    for (int q = 0; q < 9; q++) {
        off_t |= static_cast<u64>((tid >> q) & 1u) << d.lbit[q];
    }
    u64 off_r[kRows];
#pragma unroll
    for (int r = 0; r < kRows; r++) {
        u64 o = 0;
        for (int q = 0; q < 3; q++) {
            o |= static_cast<u64>((r >> q) & 1) << d.lbit[9 + q];
        }
        off_r[r] = o;
    }
    for (int w = 0; w < kPassTerms; w++) {
        sums[w * kPass12Threads + tid] = make_float2(0.f, 0.f);
    }
    auto tile_base = [&](u64 tt) {
        u64 base = 0;
        for (int q = 0; q < d.nglob; q++) {
            base |= (tt & 1u) << d.glob[q];
            tt >>= 1;
        }
        return base;
    };
    // local amplitude jj = r * 512 + tid of a tile, copied by thread tid
    auto fetch = [&](u64 tt, unsigned buf) {
        const u64 base = tile_base(tt) | off_t;
#pragma unroll
        for (int r = 0; r < kRows; r++) {
            pass_cp_async(s0 + buf * kTileBytes + (static_cast<unsigned>(r) * kPass12Threads + tid) * kAmp,
                          a + (base | off_r[r]), static_cast<int>(kAmp));
        }
    };
    const u64 stride = gridDim.x;
    u64 tile = blockIdx.x;
    if (tile < d.ntiles) {
        fetch(tile, 0);
    }
    asm volatile("cp.async.commit_group;" ::: "memory");
    for (unsigned buf = 0; tile < d.ntiles; tile += stride, buf ^= 1u) {
        if (tile + stride < d.ntiles) {
            fetch(tile + stride, buf ^ 1u);
        }
        asm volatile("cp.async.commit_group;" ::: "memory");
        asm volatile("cp.async.wait_group 1;" ::: "memory"); // this thread's copies of the tile
        unsigned char *tb = smem + buf * kTileBytes;
        if constexpr (kDF) { // in place: the copying thread converts its own amplitudes
            const double2 *raw = reinterpret_cast<const double2 *>(tb);
            float4 *tl = reinterpret_cast<float4 *>(tb);
#pragma unroll
            for (int r = 0; r < kRows; r++) {
                const unsigned jj = static_cast<unsigned>(r) * kPass12Threads + tid;
                const double2 v = raw[jj];
                const df re = df_from_bits(v.x), im = df_from_bits(v.y);
                tl[jj] = make_float4(re.hi, re.lo, im.hi, im.lo);
            }
        }
        __syncthreads();
        const u64 base = tile_base(tile);
#pragma unroll 1
        for (int w = 0; w < d.nterms; w++) {
            const PauliPassTerm &pt = d.term[w];
            const unsigned tpar = static_cast<unsigned>(__popcll(base & pt.yz)) & 1u;
            const float2 sw = sums[w * kPass12Threads + tid];
            PassAcc ac{sw.x, sw.y};
            if (pt.x == 0) {
                const unsigned st = (static_cast<unsigned>(__popc(tid & pt.yzl)) ^ tpar) & 1u;
#pragma unroll
                for (int r = 0; r < kRows; r++) {
                    const unsigned j = static_cast<unsigned>(r) * kPass12Threads + tid;
                    float sv, cv;
                    if constexpr (kDF) {
                        const float4 p = reinterpret_cast<const float4 *>(tb)[j];
                        pass_dot2(p.x, p.y, p.x, p.y, p.z, p.w, p.z, p.w, sv, cv);
                    } else {
                        const float2 p = reinterpret_cast<const float2 *>(tb)[j];
                        pass_dot2f(p.x, p.x, p.y, p.y, sv, cv);
                    }
                    pass_accumulate(ac, pass_sign(st ^ ((pt.srm >> r) & 1u)), sv, cv);
                }
            } else {
                const unsigned hb = static_cast<unsigned>(pt.hb);
                const unsigned jt = ((tid >> hb) << (hb + 1)) | (tid & ((1u << hb) - 1u));
                const unsigned st = (static_cast<unsigned>(__popc(jt & pt.yzl)) ^ tpar) & 1u;
                // Re conj(p) q = pr qr + pi qi; Im conj(p) q = pr qi - pi qr (one
                // loop per part: a branch inside would evaluate both)
                auto pairs = [&](auto im) {
#pragma unroll
                    for (int r = 0; r < kRows / 2; r++) {
                        const unsigned j = jt | pt.jr[r];
                        float sv, cv;
                        if constexpr (kDF) {
                            const float4 p = reinterpret_cast<const float4 *>(tb)[j];
                            const float4 q = reinterpret_cast<const float4 *>(tb)[j ^ pt.x];
                            if constexpr (decltype(im)::value) {
                                pass_dot2(p.x, p.y, q.z, q.w, -p.z, -p.w, q.x, q.y, sv, cv);
                            } else {
                                pass_dot2(p.x, p.y, q.x, q.y, p.z, p.w, q.z, q.w, sv, cv);
                            }
                        } else {
                            const float2 p = reinterpret_cast<const float2 *>(tb)[j];
                            const float2 q = reinterpret_cast<const float2 *>(tb)[j ^ pt.x];
                            if constexpr (decltype(im)::value) {
                                pass_dot2f(p.x, q.y, -p.y, q.x, sv, cv);
                            } else {
                                pass_dot2f(p.x, q.x, p.y, q.y, sv, cv);
                            }
                        }
                        pass_accumulate(ac, pass_sign(st ^ ((pt.srm >> r) & 1u)), sv, cv);
                    }
                };
                if (pt.im) {
                    pairs(std::true_type{});
                } else {
                    pairs(std::false_type{});
                }
            }
            sums[w * kPass12Threads + tid] = make_float2(ac.a, ac.l);
        }
        __syncthreads(); // the buffer is refilled two tiles on
    }
    asm volatile("cp.async.wait_group 0;" ::: "memory");
    double v[kPassTerms];
#pragma unroll
    for (int w = 0; w < kPassTerms; w++) {
        const float2 sw = sums[w * kPass12Threads + tid];
        v[w] = __dadd_rn(static_cast<double>(sw.x), static_cast<double>(sw.y));
    }
    block_reduce_store<kPassTerms, kPass12Threads>(v, partials);
}

template <class T> int launch_pauli_pass(cudaStream_t s, const cx<T> *sv, const PauliPass &p, double *partials) {
    const bool fast = p.t == kPassMaxTileBits;
    const size_t smem = fast ? pass12_smem<T>() : sizeof(float4) << p.t;
    auto *kern = fast ? k_pauli_pass12<T> : k_pauli_pass<T>;
    const int threads = fast ? kPass12Threads : kPassThreads;
    static bool attr = false;
    if (!attr) {
        cuda_check(cudaFuncSetAttribute(k_pauli_pass12<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        static_cast<int>(pass12_smem<T>())),
                   "k_pauli_pass12 smem attribute");
        cuda_check(cudaFuncSetAttribute(k_pauli_pass<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        static_cast<int>(sizeof(float4) << kPassMaxTileBits)),
                   "k_pauli_pass smem attribute");
        attr = true;
    }
    int per_sm = 0;
    cuda_check(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, threads, smem), "k_pauli_pass occupancy");
    const u64 cap = static_cast<u64>(LaunchGeom::sm_count()) * static_cast<u64>(per_sm < 1 ? 1 : per_sm);
    const int grid = static_cast<int>(p.ntiles < cap ? p.ntiles : cap);
    kern<<<grid, threads, smem, s>>>(sv, p, partials);
    cuda_check(cudaGetLastError(), "k_pauli_pass launch");
    note_launch();
    return grid;
}
void launch_finalize_pass(cudaStream_t s, const double *partials, int nblocks, double *out) {
    finalize<kPassTerms>(s, partials, nblocks, out);
}

// <a| Pi P |b> where Pi projects on (j & pmask) == pval (row index j):
// sum_j conj(a_j) i^ny (-1)^{|(j^x) & yz|} b_{j^x}.
template <class T>
__global__ void __launch_bounds__(kReduceThreads) k_pauli_transition(const cx<T> *__restrict__ a, const cx<T> *__restrict__ b, u64 N,
                                                                    u64 x, u64 yz, int ny4, u64 pmask, u64 pval,
                                                                    double *partials) {
    double v[2] = {0.0, 0.0};
    GRID_STRIDE(j, N) {
        if ((j & pmask) != pval) {
            continue;
        }
        const u64 k = j ^ x;
        const cx<T> p = a[j];
        const cx<T> q = b[k];
        double re = static_cast<double>(p.x) * q.x + static_cast<double>(p.y) * q.y;
        double im = static_cast<double>(p.x) * q.y - static_cast<double>(p.y) * q.x;
        if (__popcll(k & yz) & 1) {
            re = -re;
            im = -im;
        }
        switch (ny4) {
        case 0: v[0] += re; v[1] += im; break;
        case 1: v[0] -= im; v[1] += re; break;
        case 2: v[0] -= re; v[1] -= im; break;
        default: v[0] += im; v[1] -= re; break;
        }
    }
    block_reduce_store<2>(v, partials);
}
template <class T>
void reduce_pauli_transition(cudaStream_t s, const cx<T> *a, const cx<T> *b, u64 N, u64 x, u64 yz, int ny4,
                             u64 pmask, u64 pval, double *partials, double *out) {
    const int g = reduce_grid(N);
    k_pauli_transition<T><<<g, kReduceThreads, 0, s>>>(a, b, N, x, yz, ny4, pmask, pval, partials);
    cuda_check(cudaGetLastError(), "k_pauli_transition launch");
    note_launch();
    finalize<2>(s, partials, g, out);
}


// One sweep for every flip-mask group of a Pauli sum: each output amplitude
// reads its partners psi[j ^ x_g] once per group and is written once.  The
// products and sums run in double-float arithmetic on the FP32 pipe (FP64
// runs at 1/64 of it on GB300); complex128 inputs are split with integer
// operations and the result is converted once.
template <class T>
__global__ void __launch_bounds__(256) k_pauli_apply(const cx<T> *__restrict__ psi, cx<T> *__restrict__ out, u64 N,
                                                     const PauliGroupHdr *__restrict__ groups, int ngroups,
                                                     const PauliTermDF *__restrict__ terms, int nterms, int first) {
    __shared__ PauliGroupHdr sg[kApplyMaxGroups];
    __shared__ PauliTermDF st[kApplyMaxTerms];
    for (int i = static_cast<int>(threadIdx.x); i < ngroups; i += static_cast<int>(blockDim.x)) {
        sg[i] = groups[i];
    }
    for (int i = static_cast<int>(threadIdx.x); i < nterms; i += static_cast<int>(blockDim.x)) {
        st[i] = terms[i];
    }
    __syncthreads();
    GRID_STRIDE(j, N) {
        df re{0.f, 0.f}, im{0.f, 0.f};
        if (!first) {
            const cx<T> o = out[j];
            re = to_df<T>(o.x);
            im = to_df<T>(o.y);
        }
        for (int g = 0; g < ngroups; g++) {
            const u64 k = j ^ sg[g].x;
            const cx<T> q = psi[k];
            const df qr = to_df<T>(q.x), qi = to_df<T>(q.y);
            const int t0 = sg[g].tbegin, t1 = sg[g].tend;
            if (t1 - t0 == 1) { // one term: a signed real or imaginary coefficient
                const PauliTermDF &tm = st[t0];
                df c{tm.chi, tm.clo};
                if ((__popcll(k & tm.yz) & 1) != 0) {
                    c = -c;
                }
                switch (tm.ny4) {
                case 0: re = df_fma(re, c, qr); im = df_fma(im, c, qi); break;
                case 1: re = df_fma(re, -c, qi); im = df_fma(im, c, qr); break;
                case 2: re = df_fma(re, -c, qr); im = df_fma(im, -c, qi); break;
                default: re = df_fma(re, c, qi); im = df_fma(im, -c, qr); break;
                }
                continue;
            }
            df wr{0.f, 0.f}, wi{0.f, 0.f};
            for (int t = t0; t < t1; t++) {
                const PauliTermDF &tm = st[t];
                df c{tm.chi, tm.clo};
                if ((__popcll(k & tm.yz) & 1) != 0) {
                    c = -c;
                }
                switch (tm.ny4) {
                case 0: wr = wr + c; break;
                case 1: wi = wi + c; break;
                case 2: wr = wr - c; break;
                default: wi = wi - c; break;
                }
            }
            re = df_fma(df_fma(re, wr, qr), -wi, qi);
            im = df_fma(df_fma(im, wr, qi), wi, qr);
        }
        out[j] = cx<T>{from_df<T>(re), from_df<T>(im)};
    }
}
template <class T>
void launch_pauli_apply(cudaStream_t s, const cx<T> *psi, cx<T> *out, u64 N, const PauliGroupHdr *groups, int ngroups,
                        const PauliTermDF *terms, int nterms, bool first) {
    if (ngroups < 1 || ngroups > kApplyMaxGroups || nterms < 1 || nterms > kApplyMaxTerms) {
        throw std::runtime_error("Pauli-sum apply: group or term count out of range");
    }
    k_pauli_apply<T><<<grid_for(N, 256, 8), 256, 0, s>>>(psi, out, N, groups, ngroups, terms, nterms, first ? 1 : 0);
    cuda_check(cudaGetLastError(), "k_pauli_apply launch");
    note_launch();
}

// Hermitian matrix on k wires: sum over groups of Re(v^H M v).
template <class T>
__global__ void __launch_bounds__(kReduceThreads) k_expval_matrix(const cx<T> *__restrict__ a, GroupGeom g, int k, LocalOffsets lo,
                                                                 const cx<T> *__restrict__ mat, double *partials) {
    double v[1] = {0.0};
    const int D = 1 << k;
    GRID_STRIDE(q, g.ngroups) {
        const u64 b = insert_zeros(q, g.ins, g.nins);
        cx<double> x[32];
        for (int j = 0; j < D; j++) {
            const cx<T> t = a[b | lo.off[j]];
            x[j] = cx<double>{static_cast<double>(t.x), static_cast<double>(t.y)};
        }
        for (int r = 0; r < D; r++) {
            cx<double> acc{0, 0};
            for (int j = 0; j < D; j++) {
                const cx<T> m = mat[r * D + j];
                acc = cfma(cx<double>{static_cast<double>(m.x), static_cast<double>(m.y)}, x[j], acc);
            }
            v[0] += x[r].x * acc.x + x[r].y * acc.y;
        }
    }
    block_reduce_store<1>(v, partials);
}
template <class T>
void reduce_expval_matrix(cudaStream_t s, const cx<T> *sv, const GroupGeom &g, int k, const LocalOffsets &lo,
                          const cx<T> *dmat, double *partials, double *out) {
    const int grid = reduce_grid(g.ngroups);
    k_expval_matrix<T><<<grid, kReduceThreads, 0, s>>>(sv, g, k, lo, dmat, partials);
    cuda_check(cudaGetLastError(), "k_expval_matrix launch");
    note_launch();
    finalize<1>(s, partials, grid, out);
}

// CSR: Re sum_r conj(psi_r) sum_p A_rp psi_col(p)
template <class T>
__global__ void __launch_bounds__(kReduceThreads) k_expval_csr(const cx<T> *__restrict__ a, u64 N, const long long *__restrict__ ip,
                                                              const long long *__restrict__ ix,
                                                              const cx<T> *__restrict__ val, double *partials) {
    double v[1] = {0.0};
    GRID_STRIDE(r, N) {
        double ar = 0.0, ai = 0.0;
        for (long long p = ip[r]; p < ip[r + 1]; p++) {
            const cx<T> m = val[p];
            const cx<T> x = a[ix[p]];
            ar += static_cast<double>(m.x) * x.x - static_cast<double>(m.y) * x.y;
            ai += static_cast<double>(m.x) * x.y + static_cast<double>(m.y) * x.x;
        }
        const cx<T> y = a[r];
        v[0] += static_cast<double>(y.x) * ar + static_cast<double>(y.y) * ai;
    }
    block_reduce_store<1>(v, partials);
}
template <class T>
void reduce_expval_csr(cudaStream_t s, const cx<T> *sv, u64 N, const long long *indptr, const long long *indices,
                       const cx<T> *vals, double *partials, double *out) {
    const int g = reduce_grid(N);
    k_expval_csr<T><<<g, kReduceThreads, 0, s>>>(sv, N, indptr, indices, vals, partials);
    cuda_check(cudaGetLastError(), "k_expval_csr launch");
    note_launch();
    finalize<1>(s, partials, g, out);
}

template <class T>
__global__ void k_csr_apply(const cx<T> *__restrict__ a, cx<T> *__restrict__ out, u64 N, const long long *__restrict__ ip,
                            const long long *__restrict__ ix, const cx<T> *__restrict__ val) {
    GRID_STRIDE(r, N) {
        cx<T> acc{0, 0};
        for (long long p = ip[r]; p < ip[r + 1]; p++) {
            acc = cfma(val[p], a[ix[p]], acc);
        }
        out[r] = acc;
    }
}
template <class T>
void launch_csr_apply(cudaStream_t s, const cx<T> *sv, cx<T> *out, u64 N, const long long *indptr,
                      const long long *indices, const cx<T> *vals) {
    k_csr_apply<T><<<grid_for(N, 256, 8), 256, 0, s>>>(sv, out, N, indptr, indices, vals);
    cuda_check(cudaGetLastError(), "k_csr_apply launch");
    note_launch();
}

// ---------------------------------------------------------------------------
// Probabilities.
// ---------------------------------------------------------------------------
template <class T> __global__ void k_probs_all(const cx<T> *__restrict__ a, u64 N, T *__restrict__ out) {
    GRID_STRIDE(i, N) { out[i] = norm_rn(a[i]); }
}
template <class T> void launch_probs_all(cudaStream_t s, const cx<T> *sv, u64 N, T *out) {
    k_probs_all<T><<<grid_for(N, 256, 8), 256, 0, s>>>(sv, N, out);
    cuda_check(cudaGetLastError(), "k_probs_all launch");
    note_launch();
}

// Marginal over k wires: shared-memory histogram for k <= 12, global
// atomics beyond.  Output index bit (k-1-m) is wire m of the request.
// Marginal probabilities summed in the reference's order, bit for bit: one
// thread per output entry adds |a_idx|^2 (rounded as std::norm) in the
// working precision over the indices with that entry's wire bits, in
// increasing index order, starting from zero (MeasurementsLQubit.hpp:
// 142-161 for five wires and more, and probs_bitshift in
// MeasurementKernels.hpp for one to four wires, which sums in that order on
// one thread).  The serial chain per entry is what makes the rounding equal.
template <class T>
__global__ void __launch_bounds__(128) k_probs_marginal_serial(const cx<T> *__restrict__ a, MarginalGeom g, T *out) {
    const u64 j = static_cast<u64>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (j >= (u64{1} << g.k)) {
        return;
    }
    u64 base = 0;
    for (int m = 0; m < g.k; m++) {
        base |= ((j >> (g.k - 1 - m)) & 1u) << g.wb[m];
    }
    const u64 cm = g.cmask;
    T acc = 0;
    u64 sub = 0;
    do {
        const cx<T> x = a[base | sub];
        if constexpr (sizeof(T) == 8) {
            acc = __dadd_rn(acc, norm_rn(x));
        } else {
            acc = __fadd_rn(acc, norm_rn(x));
        }
        sub = (sub - cm) & cm; // next subset of the complement bits, increasing
    } while (sub != 0);
    out[j] = acc;
}
template <class T> void launch_probs_marginal_serial(cudaStream_t s, const cx<T> *sv, const MarginalGeom &g, T *out) {
    const u64 D = u64{1} << g.k;
    const unsigned grid = static_cast<unsigned>((D + 127) / 128);
    k_probs_marginal_serial<T><<<grid, 128, 0, s>>>(sv, g, out);
    cuda_check(cudaGetLastError(), "k_probs_marginal_serial launch");
    note_launch();
}

#define PLGB_INST_MEAS(T)                                                                                         \
    template void reduce_norm2<T>(cudaStream_t, const cx<T> *, u64, double *, double *);                        \
    template void reduce_inner<T>(cudaStream_t, const cx<T> *, const cx<T> *, u64, double *, double *);         \
    template void reduce_expval1<T>(cudaStream_t, const cx<T> *, u64, int, int, double *, double *);            \
    template void reduce_pauli_group<T>(cudaStream_t, const cx<T> *, u64, const PauliGroup &, double *, double *); \
    template void reduce_pauli_transition<T>(cudaStream_t, const cx<T> *, const cx<T> *, u64, u64, u64, int, u64, \
                                             u64, double *, double *);                                            \
    template void reduce_expval_matrix<T>(cudaStream_t, const cx<T> *, const GroupGeom &, int, const LocalOffsets &, \
                                          const cx<T> *, double *, double *);                                     \
    template void reduce_expval_csr<T>(cudaStream_t, const cx<T> *, u64, const long long *, const long long *,   \
                                       const cx<T> *, double *, double *);                                        \
    template void launch_csr_apply<T>(cudaStream_t, const cx<T> *, cx<T> *, u64, const long long *,              \
                                      const long long *, const cx<T> *);                                          \
    template void launch_pauli_apply<T>(cudaStream_t, const cx<T> *, cx<T> *, u64, const PauliGroupHdr *, int,    \
                                        const PauliTermDF *, int, bool);                                          \
    template void launch_probs_all<T>(cudaStream_t, const cx<T> *, u64, T *);                                    \
    template void launch_probs_marginal_serial<T>(cudaStream_t, const cx<T> *, const MarginalGeom &, T *);     \
    template int launch_pauli_pass<T>(cudaStream_t, const cx<T> *, const PauliPass &, double *);

PLGB_INST_MEAS(float)
PLGB_INST_MEAS(double)

} // namespace plgb
