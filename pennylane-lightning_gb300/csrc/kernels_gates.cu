// Gate kernels (sm_103a).  Every kernel is memory-streaming: one pass over the
// amplitudes it touches, 128-bit (c128) / 64-bit (c64) accesses, grid-stride
// loops over a grid that is a multiple of the SM count.  Coefficients are
// formed on the host in the working precision (host_statevector.cpp) and passed
// by value, so kernels only multiply and add.
//
// Reference semantics: pennylane_lightning/core/simulators/lightning_qubit/
// gates/cpu_kernels/GateImplementationsLM.hpp (applyNC1 :653-703, applyNC2
// :1325-1385, applyNCN :408-440, applyMultiRZ :1989-2043, applyPauliRot
// :577-629).
#include "kernels.hpp"

namespace plgb {

// ---------------------------------------------------------------------------
// One-target kernels.
// ---------------------------------------------------------------------------
template <class T, int MODE>
__device__ __forceinline__ void op1(cx<T> *__restrict__ a, u64 i0, u64 i1, const Mat1<T> &m) {
    if constexpr (MODE == M1_PHASE1) {
        a[i1] = m.m[3] * a[i1];
    } else if constexpr (MODE == M1_NEG1) {
        const cx<T> v = a[i1];
        a[i1] = cx<T>{-v.x, -v.y};
    } else if constexpr (MODE == M1_SWAP) {
        const cx<T> v0 = a[i0];
        const cx<T> v1 = a[i1];
        a[i0] = v1;
        a[i1] = v0;
    } else {
        const cx<T> v0 = a[i0];
        const cx<T> v1 = a[i1];
        cx<T> r0, r1;
        if constexpr (MODE == M1_DENSE) {
            r0 = cfma(m.m[1], v1, m.m[0] * v0);
            r1 = cfma(m.m[3], v1, m.m[2] * v0);
        } else if constexpr (MODE == M1_REAL) {
            // real 2x2: RY, Hadamard
            r0 = cx<T>{m.m[0].x * v0.x + m.m[1].x * v1.x, m.m[0].x * v0.y + m.m[1].x * v1.y};
            r1 = cx<T>{m.m[2].x * v0.x + m.m[3].x * v1.x, m.m[2].x * v0.y + m.m[3].x * v1.y};
        } else if constexpr (MODE == M1_RXF) {
            // [[c, i s],[i s, c]] with c = m00.x, s = m01.y (RX family)
            const T c = m.m[0].x, s = m.m[1].y;
            r0 = cx<T>{c * v0.x - s * v1.y, c * v0.y + s * v1.x};
            r1 = cx<T>{c * v1.x - s * v0.y, c * v1.y + s * v0.x};
        } else if constexpr (MODE == M1_DIAG) {
            r0 = m.m[0] * v0;
            r1 = m.m[3] * v1;
        } else { // M1_ANTI
            r0 = m.m[1] * v1;
            r1 = m.m[2] * v0;
        }
        a[i0] = r0;
        a[i1] = r1;
    }
}

template <class T, int MODE>
__global__ void __launch_bounds__(256) k_1q(cx<T> *__restrict__ a, GroupGeom g, u64 o0, u64 o1, Mat1<T> m) {
    // A "pair" gate: groups are enumerated with zero bits inserted at g.ins;
    // the two mixed amplitudes are base|o0 and base|o1 (for a one-wire gate
    // o0 = 0 and o1 = the target bit; SWAP-like gates use |01>, |10>).
    const u64 stride = static_cast<u64>(gridDim.x) * blockDim.x;
    u64 k = static_cast<u64>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (g.nins == 1) {
        // uncontrolled one-wire fast path: two pairs in flight per thread
        const int tb = g.ins[0];
        for (; k + stride < g.ngroups; k += 2 * stride) {
            const u64 b0 = insert_zero(k, tb);
            const u64 b1 = insert_zero(k + stride, tb);
            op1<T, MODE>(a, b0 | o0, b0 | o1, m);
            op1<T, MODE>(a, b1 | o0, b1 | o1, m);
        }
        if (k < g.ngroups) {
            const u64 b0 = insert_zero(k, tb);
            op1<T, MODE>(a, b0 | o0, b0 | o1, m);
        }
        return;
    }
    for (; k < g.ngroups; k += stride) {
        const u64 b = insert_zeros(k, g.ins, g.nins) | g.cval;
        op1<T, MODE>(a, b | o0, b | o1, m);
    }
}

template <class T>
void launch_1q(cudaStream_t s, cx<T> *sv, const GroupGeom &g, u64 o0, u64 o1, int mode, const Mat1<T> &m) {
    constexpr int B = 256;
    const unsigned grid = grid_for(g.ngroups, B, 8);
    switch (mode) {
    case M1_DENSE: k_1q<T, M1_DENSE><<<grid, B, 0, s>>>(sv, g, o0, o1, m); break;
    case M1_REAL: k_1q<T, M1_REAL><<<grid, B, 0, s>>>(sv, g, o0, o1, m); break;
    case M1_RXF: k_1q<T, M1_RXF><<<grid, B, 0, s>>>(sv, g, o0, o1, m); break;
    case M1_DIAG: k_1q<T, M1_DIAG><<<grid, B, 0, s>>>(sv, g, o0, o1, m); break;
    case M1_PHASE1: k_1q<T, M1_PHASE1><<<grid, B, 0, s>>>(sv, g, o0, o1, m); break;
    case M1_SWAP: k_1q<T, M1_SWAP><<<grid, B, 0, s>>>(sv, g, o0, o1, m); break;
    case M1_ANTI: k_1q<T, M1_ANTI><<<grid, B, 0, s>>>(sv, g, o0, o1, m); break;
    case M1_NEG1: k_1q<T, M1_NEG1><<<grid, B, 0, s>>>(sv, g, o0, o1, m); break;
    default: throw std::runtime_error("launch_1q: bad mode");
    }
    cuda_check(cudaGetLastError(), "k_1q launch");
    note_launch();
}

// ---------------------------------------------------------------------------
// Two-target kernel: dense 4x4 (row-major, local index bit1 = first wire).
// ---------------------------------------------------------------------------
template <class T, bool DIAG>
__global__ void __launch_bounds__(256) k_2q(cx<T> *__restrict__ a, GroupGeom g, u64 off1, u64 off0, Mat2<T> m) {
    const u64 stride = static_cast<u64>(gridDim.x) * blockDim.x;
    for (u64 k = static_cast<u64>(blockIdx.x) * blockDim.x + threadIdx.x; k < g.ngroups; k += stride) {
        const u64 b = insert_zeros(k, g.ins, g.nins) | g.cval;
        const u64 ix[4] = {b, b | off0, b | off1, b | off1 | off0};
        if constexpr (DIAG) {
#pragma unroll
            for (int r = 0; r < 4; r++) {
                a[ix[r]] = m.m[5 * r] * a[ix[r]];
            }
        } else {
            cx<T> v[4];
#pragma unroll
            for (int r = 0; r < 4; r++) {
                v[r] = a[ix[r]];
            }
#pragma unroll
            for (int r = 0; r < 4; r++) {
                cx<T> acc = m.m[4 * r] * v[0];
                acc = cfma(m.m[4 * r + 1], v[1], acc);
                acc = cfma(m.m[4 * r + 2], v[2], acc);
                acc = cfma(m.m[4 * r + 3], v[3], acc);
                a[ix[r]] = acc;
            }
        }
    }
}

template <class T>
void launch_2q(cudaStream_t s, cx<T> *sv, const GroupGeom &g, int bit_hi_local, int bit_lo_local, bool diag,
               const Mat2<T> &m) {
    constexpr int B = 256;
    const unsigned grid = grid_for(g.ngroups, B, 8);
    const u64 off1 = u64{1} << bit_hi_local, off0 = u64{1} << bit_lo_local;
    if (diag) {
        k_2q<T, true><<<grid, B, 0, s>>>(sv, g, off1, off0, m);
    } else {
        k_2q<T, false><<<grid, B, 0, s>>>(sv, g, off1, off0, m);
    }
    cuda_check(cudaGetLastError(), "k_2q launch");
    note_launch();
}

// ---------------------------------------------------------------------------
// k-target dense kernel, 3 <= k <= 5: one group per thread, matrix in smem.
// ---------------------------------------------------------------------------
template <class T, int K>
__global__ void __launch_bounds__(128) k_kq(cx<T> *__restrict__ a, GroupGeom g, LocalOffsets lo,
                                            const cx<T> *__restrict__ mat) {
    constexpr int D = 1 << K;
    __shared__ cx<T> sm[D * D];
    for (int i = threadIdx.x; i < D * D; i += blockDim.x) {
        sm[i] = mat[i];
    }
    __syncthreads();
    const u64 stride = static_cast<u64>(gridDim.x) * blockDim.x;
    for (u64 k = static_cast<u64>(blockIdx.x) * blockDim.x + threadIdx.x; k < g.ngroups; k += stride) {
        const u64 b = insert_zeros(k, g.ins, g.nins) | g.cval;
        cx<T> v[D];
#pragma unroll
        for (int j = 0; j < D; j++) {
            v[j] = a[b | lo.off[j]];
        }
#pragma unroll 1
        for (int r = 0; r < D; r++) {
            cx<T> acc{0, 0};
#pragma unroll
            for (int j = 0; j < D; j++) {
                acc = cfma(sm[r * D + j], v[j], acc);
            }
            a[b | lo.off[r]] = acc;
        }
    }
}

// k-target dense kernel for 6 <= k <= 12: one CTA per group, the group and the
// matrix rows are read through smem / L2.
template <class T>
__global__ void __launch_bounds__(256) k_kq_cta(cx<T> *__restrict__ a, GroupGeom g, int k, const u64 *__restrict__ loc,
                                                const cx<T> *__restrict__ mat) {
    extern __shared__ unsigned char smraw[];
    cx<T> *v = reinterpret_cast<cx<T> *>(smraw);
    const int D = 1 << k;
    for (u64 grp = blockIdx.x; grp < g.ngroups; grp += gridDim.x) {
        const u64 b = insert_zeros(grp, g.ins, g.nins) | g.cval;
        for (int j = threadIdx.x; j < D; j += blockDim.x) {
            v[j] = a[b | loc[j]];
        }
        __syncthreads();
        for (int r = threadIdx.x; r < D; r += blockDim.x) {
            cx<T> acc{0, 0};
            const cx<T> *row = mat + static_cast<u64>(r) * D;
            for (int j = 0; j < D; j++) {
                acc = cfma(row[j], v[j], acc);
            }
            a[b | loc[r]] = acc;
        }
        __syncthreads();
    }
}

template <class T>
void launch_kq(cudaStream_t s, cx<T> *sv, const GroupGeom &g, int k, const LocalOffsets &lo, const cx<T> *dmat,
               const u64 *dloc) {
    switch (k) {
    case 3: k_kq<T, 3><<<grid_for(g.ngroups, 128, 8), 128, 0, s>>>(sv, g, lo, dmat); break;
    case 4: k_kq<T, 4><<<grid_for(g.ngroups, 128, 8), 128, 0, s>>>(sv, g, lo, dmat); break;
    case 5: k_kq<T, 5><<<grid_for(g.ngroups, 128, 4), 128, 0, s>>>(sv, g, lo, dmat); break;
    default: {
        const size_t smem = sizeof(cx<T>) << k;
        if (smem > 48 * 1024) {
            cuda_check(cudaFuncSetAttribute(k_kq_cta<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                            static_cast<int>(smem)),
                       "k_kq_cta smem attribute");
        }
        const u64 nb = g.ngroups < u64{65535} ? g.ngroups : u64{65535};
        k_kq_cta<T><<<static_cast<unsigned>(nb), 256, smem, s>>>(sv, g, k, dloc, dmat);
    }
    }
    cuda_check(cudaGetLastError(), "k_kq launch");
    note_launch();
}

// ---------------------------------------------------------------------------
// Diagonal on k target bits (k <= 10), with controls; diag values in global.
// ---------------------------------------------------------------------------
template <class T>
__global__ void __launch_bounds__(256) k_diag(cx<T> *__restrict__ a, u64 N, u64 cmask, u64 cval, int k, TBits tb,
                                              const cx<T> *__restrict__ d) {
    const u64 stride = static_cast<u64>(gridDim.x) * blockDim.x;
    for (u64 i = static_cast<u64>(blockIdx.x) * blockDim.x + threadIdx.x; i < N; i += stride) {
        if ((i & cmask) != cval) {
            continue;
        }
        unsigned j = 0;
        for (int m = 0; m < k; m++) {
            j = (j << 1) | static_cast<unsigned>((i >> tb.b[m]) & 1U);
        }
        a[i] = d[j] * a[i];
    }
}

template <class T>
void launch_diag(cudaStream_t s, cx<T> *sv, u64 N, u64 cmask, u64 cval, int k, const TBits &tb, const cx<T> *dd) {
    k_diag<T><<<grid_for(N, 256, 8), 256, 0, s>>>(sv, N, cmask, cval, k, tb, dd);
    cuda_check(cudaGetLastError(), "k_diag launch");
    note_launch();
}

// Parity phase: a[i] *= s[popcount(i & pmask) & 1] where (i & cmask) == cval
// (MultiRZ, LM:1989-2043).  With `zero_outside` the non-control subspace is
// zeroed (controlled MultiRZ generator, LM:2900-2940).
template <class T>
__global__ void __launch_bounds__(256) k_parity(cx<T> *__restrict__ a, u64 N, u64 pmask, u64 cmask, u64 cval,
                                                cx<T> s0, cx<T> s1, int zero_outside) {
    const u64 stride = static_cast<u64>(gridDim.x) * blockDim.x;
    for (u64 i = static_cast<u64>(blockIdx.x) * blockDim.x + threadIdx.x; i < N; i += stride) {
        if ((i & cmask) != cval) {
            if (zero_outside) {
                a[i] = cx<T>{0, 0};
            }
            continue;
        }
        const cx<T> f = (__popcll(i & pmask) & 1) ? s1 : s0;
        a[i] = f * a[i];
    }
}

template <class T>
void launch_parity(cudaStream_t s, cx<T> *sv, u64 N, u64 pmask, u64 cmask, u64 cval, cx<T> s0, cx<T> s1,
                   bool zero_outside) {
    k_parity<T><<<grid_for(N, 256, 8), 256, 0, s>>>(sv, N, pmask, cmask, cval, s0, s1, zero_outside ? 1 : 0);
    cuda_check(cudaGetLastError(), "k_parity launch");
    note_launch();
}

// PauliRot (LM:577-629): pairs (i, i ^ mask_xy), i < partner.
template <class T>
__global__ void __launch_bounds__(256) k_pauli_rot(cx<T> *__restrict__ a, u64 half, int hb, u64 mxy, u64 my, u64 mz,
                                                   int cmy, T c, cx<T> s) {
    const cx<T> I{0, 1};
    const cx<T> sines[4] = {s, I * s, cx<T>{-s.x, -s.y}, cx<T>{-(I * s).x, -(I * s).y}};
    const u64 stride = static_cast<u64>(gridDim.x) * blockDim.x;
    for (u64 k = static_cast<u64>(blockIdx.x) * blockDim.x + threadIdx.x; k < half; k += stride) {
        const u64 i0 = insert_zero(k, hb); // highest flipped bit clear: i0 < i1
        const u64 i1 = i0 ^ mxy;
        const int cy = __popcll(i0 & my) * 2;
        const int cz = __popcll(i0 & mz) * 2;
        const int s0 = cz + cmy * 3 - cy;
        const int s1 = cz + cmy + cy;
        const cx<T> v0 = a[i0];
        const cx<T> v1 = a[i1];
        a[i0] = cfma(sines[s0 % 4], v1, c * v0);
        a[i1] = cfma(sines[s1 % 4], v0, c * v1);
    }
}

template <class T>
void launch_pauli_rot(cudaStream_t s, cx<T> *sv, int n, u64 mxy, u64 my, u64 mz, T c, cx<T> sn) {
    const u64 half = (u64{1} << n) >> 1;
    const int hb = 63 - __builtin_clzll(mxy);
    k_pauli_rot<T><<<grid_for(half, 256, 8), 256, 0, s>>>(sv, half, hb, mxy, my, mz, __builtin_popcountll(my), c, sn);
    cuda_check(cudaGetLastError(), "k_pauli_rot launch");
    note_launch();
}

// ---------------------------------------------------------------------------
// Elementwise helpers.
// ---------------------------------------------------------------------------
template <class T>
__global__ void k_zero_outside(cx<T> *__restrict__ a, u64 N, u64 cmask, u64 cval) {
    const u64 stride = static_cast<u64>(gridDim.x) * blockDim.x;
    for (u64 i = static_cast<u64>(blockIdx.x) * blockDim.x + threadIdx.x; i < N; i += stride) {
        if ((i & cmask) != cval) {
            a[i] = cx<T>{0, 0};
        }
    }
}
template <class T> void launch_zero_outside(cudaStream_t s, cx<T> *sv, u64 N, u64 cmask, u64 cval) {
    k_zero_outside<T><<<grid_for(N, 256, 8), 256, 0, s>>>(sv, N, cmask, cval);
    cuda_check(cudaGetLastError(), "k_zero_outside launch");
    note_launch();
}

template <class T> __global__ void k_scale(cx<T> *__restrict__ a, u64 N, cx<T> f, u64 cmask, u64 cval) {
    const u64 stride = static_cast<u64>(gridDim.x) * blockDim.x;
    for (u64 i = static_cast<u64>(blockIdx.x) * blockDim.x + threadIdx.x; i < N; i += stride) {
        if ((i & cmask) == cval) {
            a[i] = f * a[i];
        }
    }
}
template <class T> void launch_scale(cudaStream_t s, cx<T> *sv, u64 N, cx<T> f, u64 cmask, u64 cval) {
    k_scale<T><<<grid_for(N, 256, 8), 256, 0, s>>>(sv, N, f, cmask, cval);
    cuda_check(cudaGetLastError(), "k_scale launch");
    note_launch();
}

// y += f * x
template <class T> __global__ void k_axpy(cx<T> *__restrict__ y, const cx<T> *__restrict__ x, u64 N, cx<T> f) {
    const u64 stride = static_cast<u64>(gridDim.x) * blockDim.x;
    for (u64 i = static_cast<u64>(blockIdx.x) * blockDim.x + threadIdx.x; i < N; i += stride) {
        y[i] = cfma(f, x[i], y[i]);
    }
}
template <class T> void launch_axpy(cudaStream_t s, cx<T> *y, const cx<T> *x, u64 N, cx<T> f) {
    k_axpy<T><<<grid_for(N, 256, 8), 256, 0, s>>>(y, x, N, f);
    cuda_check(cudaGetLastError(), "k_axpy launch");
    note_launch();
}

// Scatter a 2^k sub-state onto the subspace where every other wire is 0
// (StateVectorLQubit.hpp:971-1036 setStateVector(state, wires)).
template <class T>
__global__ void k_scatter_sub(cx<T> *__restrict__ a, const cx<T> *__restrict__ sub, u64 D, const u64 *__restrict__ loc) {
    const u64 stride = static_cast<u64>(gridDim.x) * blockDim.x;
    for (u64 j = static_cast<u64>(blockIdx.x) * blockDim.x + threadIdx.x; j < D; j += stride) {
        a[loc[j]] = sub[j];
    }
}
template <class T> void launch_scatter_sub(cudaStream_t s, cx<T> *sv, const cx<T> *sub, u64 D, const u64 *loc) {
    k_scatter_sub<T><<<grid_for(D, 256, 8), 256, 0, s>>>(sv, sub, D, loc);
    cuda_check(cudaGetLastError(), "k_scatter_sub launch");
    note_launch();
}

// Sparse local operator on k wires (CSR, applyNCMultiQubitSparseOp LM:505-560),
// one group per thread, k <= 5.
template <class T>
__global__ void __launch_bounds__(128) k_sparse_local(cx<T> *__restrict__ a, GroupGeom g, LocalOffsets lo, int k,
                                                      const long long *__restrict__ indptr,
                                                      const long long *__restrict__ indices,
                                                      const cx<T> *__restrict__ vals) {
    const int D = 1 << k;
    const u64 stride = static_cast<u64>(gridDim.x) * blockDim.x;
    for (u64 q = static_cast<u64>(blockIdx.x) * blockDim.x + threadIdx.x; q < g.ngroups; q += stride) {
        const u64 b = insert_zeros(q, g.ins, g.nins) | g.cval;
        cx<T> v[32];
        for (int j = 0; j < D; j++) {
            v[j] = a[b | lo.off[j]];
        }
        for (int r = 0; r < D; r++) {
            cx<T> acc{0, 0};
            for (long long p = indptr[r]; p < indptr[r + 1]; p++) {
                acc = cfma(vals[p], v[indices[p]], acc);
            }
            a[b | lo.off[r]] = acc;
        }
    }
}
template <class T>
void launch_sparse_local(cudaStream_t s, cx<T> *sv, const GroupGeom &g, const LocalOffsets &lo, int k,
                         const long long *indptr, const long long *indices, const cx<T> *vals) {
    k_sparse_local<T><<<grid_for(g.ngroups, 128, 8), 128, 0, s>>>(sv, g, lo, k, indptr, indices, vals);
    cuda_check(cudaGetLastError(), "k_sparse_local launch");
    note_launch();
}

#define PLGB_INST_GATES(T)                                                                                        \
    template void launch_1q<T>(cudaStream_t, cx<T> *, const GroupGeom &, u64, u64, int, const Mat1<T> &);             \
    template void launch_2q<T>(cudaStream_t, cx<T> *, const GroupGeom &, int, int, bool, const Mat2<T> &);       \
    template void launch_kq<T>(cudaStream_t, cx<T> *, const GroupGeom &, int, const LocalOffsets &,               \
                               const cx<T> *, const u64 *);                                                       \
    template void launch_diag<T>(cudaStream_t, cx<T> *, u64, u64, u64, int, const TBits &, const cx<T> *);        \
    template void launch_parity<T>(cudaStream_t, cx<T> *, u64, u64, u64, u64, cx<T>, cx<T>, bool);               \
    template void launch_pauli_rot<T>(cudaStream_t, cx<T> *, int, u64, u64, u64, T, cx<T>);                      \
    template void launch_zero_outside<T>(cudaStream_t, cx<T> *, u64, u64, u64);                                   \
    template void launch_scale<T>(cudaStream_t, cx<T> *, u64, cx<T>, u64, u64);                                  \
    template void launch_axpy<T>(cudaStream_t, cx<T> *, const cx<T> *, u64, cx<T>);                              \
    template void launch_scatter_sub<T>(cudaStream_t, cx<T> *, const cx<T> *, u64, const u64 *);                 \
    template void launch_sparse_local<T>(cudaStream_t, cx<T> *, const GroupGeom &, const LocalOffsets &, int,     \
                                         const long long *, const long long *, const cx<T> *);

PLGB_INST_GATES(float)
PLGB_INST_GATES(double)

} // namespace plgb
