// Shared device/host definitions for the GB300 state-vector kernels.
//
// Amplitude layout in HBM: one contiguous array of 2^n interleaved (re, im)
// pairs of T (float for complex64, double for complex128), 256-byte aligned
// by cudaMalloc.  Wire w is bit (n-1-w) of the amplitude index, so a HIGH
// wire number is a LOW bit with a small stride (lightning.qubit convention,
// pennylane_lightning/core/simulators/lightning_qubit/StateVectorLQubit.hpp:950).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <stdexcept>
#include <string>

namespace plgb {

using u64 = unsigned long long;
using u32 = unsigned int;

template <class T> struct alignas(2 * sizeof(T)) cx {
    T x, y;
};

template <class T> __host__ __device__ inline cx<T> mk(T a, T b) { return cx<T>{a, b}; }
template <class T> __host__ __device__ inline cx<T> operator+(cx<T> a, cx<T> b) {
    return {a.x + b.x, a.y + b.y};
}
template <class T> __host__ __device__ inline cx<T> operator-(cx<T> a, cx<T> b) {
    return {a.x - b.x, a.y - b.y};
}
template <class T> __host__ __device__ inline cx<T> operator*(cx<T> a, cx<T> b) {
    return {a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x};
}
template <class T> __host__ __device__ inline cx<T> operator*(T s, cx<T> a) {
    return {s * a.x, s * a.y};
}
template <class T> __host__ __device__ inline cx<T> conj(cx<T> a) { return {a.x, -a.y}; }
// acc + a * b
template <class T> __host__ __device__ inline cx<T> cfma(cx<T> a, cx<T> b, cx<T> acc) {
    return {acc.x + a.x * b.x - a.y * b.y, acc.y + a.x * b.y + a.y * b.x};
}

#if defined(__CUDACC__)
// |psi_i|^2 rounded exactly as std::norm does without contraction (two
// products, one sum), so the distribution a seeded sampler consumes is
// bit-identical to the reference's.
__device__ __forceinline__ double norm_rn(cx<double> x) { return __dadd_rn(__dmul_rn(x.x, x.x), __dmul_rn(x.y, x.y)); }
__device__ __forceinline__ float norm_rn(cx<float> x) { return __fadd_rn(__fmul_rn(x.x, x.x), __fmul_rn(x.y, x.y)); }
#endif

// Insert a zero bit at each of the `nins` ascending positions `ins`.
__host__ __device__ inline u64 insert_zeros(u64 k, const int *ins, int nins) {
    for (int i = 0; i < nins; i++) {
        const int p = ins[i];
        const u64 lo = k & ((u64{1} << p) - 1);
        k = ((k >> p) << (p + 1)) | lo;
    }
    return k;
}
__host__ __device__ inline u64 insert_zero(u64 k, int p) {
    const u64 lo = k & ((u64{1} << p) - 1);
    return ((k >> p) << (p + 1)) | lo;
}

#define PLGB_MAX_INS 40

// Group geometry shared by the gate kernels: a group is the 2^k amplitudes a
// k-target operation mixes.  Groups are enumerated by a compact counter into
// which zero bits are inserted at every target and control position; the
// control values are then or'ed in.
struct GroupGeom {
    u64 ngroups;
    u64 cval;  // control-value bits (already placed)
    int nins;  // number of inserted bits (targets + controls)
    int ins[PLGB_MAX_INS];
};

// Monotonic count of kernel launches issued by this library (all launchers
// call note_launch() after a successful launch).
void note_launch();
unsigned long long launch_count();

inline void cuda_check(cudaError_t e, const char *what) {
    if (e != cudaSuccess) {
        throw std::runtime_error(std::string(what) + ": " + cudaGetErrorString(e));
    }
}

// Grid sizing: a multiple of the SM count (152 on GB300) times resident
// blocks per SM, capped by the work.
struct LaunchGeom {
    static int sm_count();
};

inline unsigned grid_for(u64 work, int block, int per_sm = 8) {
    const u64 want = (work + static_cast<u64>(block) - 1) / static_cast<u64>(block);
    const u64 cap = static_cast<u64>(LaunchGeom::sm_count()) * static_cast<u64>(per_sm);
    const u64 g = want < cap ? want : cap;
    return static_cast<unsigned>(g < 1 ? 1 : g);
}

} // namespace plgb
