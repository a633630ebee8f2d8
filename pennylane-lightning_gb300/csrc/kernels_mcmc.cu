// Metropolis-Hastings sampling on the device (generate_mcmc_samples,
// MeasurementsLQubit.hpp:551-594 and metropolis_step :740-770, transition
// kernels TransitionKernels.hpp).
//
// The chain itself is serial, but every random number it consumes is drawn
// on the host from std::mt19937 in the reference's order (the draws do not
// depend on the state), so the device work splits into:
//   - non-zero-random kernel: count the amplitudes above epsilon per chunk,
//     then resolve every drawn rank to its amplitude index and log-probability
//     in parallel (one warp per step: binary search over the chunk prefix,
//     ballot scan inside the chunk); only the accept / reject decisions run
//     serially, over staged per-step values;
//   - local bit-flip kernel: one thread walks the chain (each proposal
//     depends on the current index).
// The |psi|^2 rounding (norm_rn) and the comparisons follow the reference
// (std::min<T>(1, x) returns x only when x < 1; a NaN ratio accepts).
#include "kernels.hpp"

namespace plgb {

namespace {

template <class T> __device__ __forceinline__ T log_t(T x) {
    if constexpr (sizeof(T) == 4) {
        return logf(x);
    } else {
        return log(x);
    }
}
template <class T> __device__ __forceinline__ T exp_t(T x) {
    if constexpr (sizeof(T) == 4) {
        return expf(x);
    } else {
        return exp(x);
    }
}
// std::abs(std::complex<T>) > epsilon (NonZeroRandomTransitionKernel)
template <class T> __device__ __forceinline__ bool above_eps(cx<T> v, T eps) {
    if constexpr (sizeof(T) == 4) {
        return hypotf(v.x, v.y) > eps;
    } else {
        return hypot(v.x, v.y) > eps;
    }
}
template <class T> __device__ __forceinline__ T plog_of(cx<T> v) { return log_t<T>(norm_rn(v)); }
// alph = std::min<T>(1, exp(trans - init)); accept when ran < alph
template <class T> __device__ __forceinline__ bool accept(T trans_plog, T init_plog, T ran) {
    const T x = exp_t<T>(trans_plog - init_plog);
    const T alph = (x < T(1)) ? x : T(1);
    return ran < alph;
}

} // namespace

template <class T>
__global__ void __launch_bounds__(256) k_nz_count(const cx<T> *__restrict__ a, u64 N, T eps, u64 nchunks,
                                                  unsigned *__restrict__ counts) {
    const int lane = static_cast<int>(threadIdx.x & 31u);
    const u64 nwarps = (static_cast<u64>(gridDim.x) * blockDim.x) >> 5;
    for (u64 c = (static_cast<u64>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5; c < nchunks; c += nwarps) {
        const u64 b = c * kMcmcChunk;
        const u64 e = b + kMcmcChunk < N ? b + kMcmcChunk : N;
        unsigned cnt = 0;
        for (u64 i = b + static_cast<u64>(lane); i < e; i += 32) {
            cnt += above_eps(a[i], eps) ? 1u : 0u;
        }
#pragma unroll
        for (int m = 16; m > 0; m >>= 1) {
            cnt += __shfl_xor_sync(0xffffffffu, cnt, m);
        }
        if (lane == 0) {
            counts[c] = cnt;
        }
    }
}

// One warp per step: the amplitude index of non-zero number rank[s] (in
// index order) and its log-probability.  prefix[c] = non-zero amplitudes in
// the chunks before c; prefix[nchunks] = total > every rank.
template <class T>
__global__ void __launch_bounds__(256) k_nz_select(const cx<T> *__restrict__ a, u64 N, T eps,
                                                   const u64 *__restrict__ prefix, u64 nchunks,
                                                   const u64 *__restrict__ rank, u64 steps, u64 *__restrict__ tidx,
                                                   T *__restrict__ tplog) {
    const int lane = static_cast<int>(threadIdx.x & 31u);
    const u64 nwarps = (static_cast<u64>(gridDim.x) * blockDim.x) >> 5;
    for (u64 s = (static_cast<u64>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5; s < steps; s += nwarps) {
        const u64 k = rank[s];
        u64 lo = 0, hi = nchunks - 1; // last chunk whose prefix is <= k
        while (lo < hi) {
            const u64 mid = (lo + hi + 1) >> 1;
            if (prefix[mid] <= k) {
                lo = mid;
            } else {
                hi = mid - 1;
            }
        }
        u64 r = k - prefix[lo];
        const u64 b = lo * kMcmcChunk;
        const u64 e = b + kMcmcChunk < N ? b + kMcmcChunk : N;
        u64 found = e; // stays e only if the counts were inconsistent
        for (u64 base = b; base < e; base += 32) {
            const u64 i = base + static_cast<u64>(lane);
            const bool nz = i < e && above_eps(a[i], eps);
            unsigned m = __ballot_sync(0xffffffffu, nz);
            const u64 pc = static_cast<u64>(__popc(m));
            if (r < pc) {
                for (u64 q = 0; q < r; q++) {
                    m &= m - 1u;
                }
                found = base + static_cast<u64>(__ffs(static_cast<int>(m)) - 1);
                break;
            }
            r -= pc;
        }
        if (lane == 0) {
            const u64 idx = found < e ? found : b;
            tidx[s] = idx;
            tplog[s] = plog_of(a[idx]);
        }
    }
}

// Accept / reject over per-step proposals, staged through shared memory by
// the whole block; one thread decides.  out[s - burnin] = chain index.
template <class T>
__global__ void __launch_bounds__(256) k_mcmc_chain_nz(const cx<T> *__restrict__ a, const u64 *__restrict__ tidx,
                                                       const T *__restrict__ tplog, const T *__restrict__ ran,
                                                       u64 steps, u64 burnin, u64 *__restrict__ out) {
    constexpr int kStage = 1024;
    __shared__ u64 s_idx[kStage];
    __shared__ T s_plog[kStage];
    __shared__ T s_ran[kStage];
    __shared__ u64 s_out[kStage];
    u64 cur = 0;
    T cur_plog = plog_of(a[0]);
    for (u64 s0 = 0; s0 < steps; s0 += kStage) {
        const int len = static_cast<int>(steps - s0 < kStage ? steps - s0 : kStage);
        for (int j = static_cast<int>(threadIdx.x); j < len; j += static_cast<int>(blockDim.x)) {
            s_idx[j] = tidx[s0 + static_cast<u64>(j)];
            s_plog[j] = tplog[s0 + static_cast<u64>(j)];
            s_ran[j] = ran[s0 + static_cast<u64>(j)];
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            for (int j = 0; j < len; j++) {
                if (accept<T>(s_plog[j], cur_plog, s_ran[j])) {
                    cur = s_idx[j];
                    cur_plog = s_plog[j];
                }
                s_out[j] = cur;
            }
        }
        __syncthreads();
        for (int j = static_cast<int>(threadIdx.x); j < len; j += static_cast<int>(blockDim.x)) {
            const u64 s = s0 + static_cast<u64>(j);
            if (s >= burnin) {
                out[s - burnin] = s_out[j];
            }
        }
        __syncthreads();
    }
}

// Local kernel: flip bit site[s] of the current index when value[s] differs
// from it (the reference tests the bit of the index truncated to 32 bits).
template <class T>
__global__ void k_mcmc_chain_local(const cx<T> *__restrict__ a, const unsigned char *__restrict__ site,
                                   const unsigned char *__restrict__ value, const T *__restrict__ ran, u64 steps,
                                   u64 burnin, u64 *__restrict__ out) {
    if (threadIdx.x != 0 || blockIdx.x != 0) {
        return;
    }
    u64 cur = 0;
    T cur_plog = plog_of(a[0]);
    for (u64 s = 0; s < steps; s++) {
        const unsigned st = site[s];
        const unsigned bit = (static_cast<unsigned>(cur) >> st) & 1u;
        u64 trans = cur;
        T trans_plog = cur_plog;
        if (value[s] != bit) {
            trans = bit == 0 ? cur + (u64{1} << st) : cur - (u64{1} << st);
            trans_plog = plog_of(a[trans]);
        }
        if (accept<T>(trans_plog, cur_plog, ran[s])) {
            cur = trans;
            cur_plog = trans_plog;
        }
        if (s >= burnin) {
            out[s - burnin] = cur;
        }
    }
}

// samples[s * n + (n - 1 - j)] = bit j of index s
__global__ void k_index_bits(const u64 *__restrict__ idx, u64 shots, int n, long long *__restrict__ out) {
    const u64 total = shots * static_cast<u64>(n);
    for (u64 t = static_cast<u64>(blockIdx.x) * blockDim.x + threadIdx.x; t < total;
         t += static_cast<u64>(gridDim.x) * blockDim.x) {
        const u64 s = t / static_cast<u64>(n);
        const int p = static_cast<int>(t - s * static_cast<u64>(n));
        out[t] = static_cast<long long>((idx[s] >> (n - 1 - p)) & 1u);
    }
}

template <class T>
void launch_nz_count(cudaStream_t s, const cx<T> *sv, u64 N, T eps, u64 nchunks, unsigned *counts) {
    const u64 blocks = (nchunks + 7) / 8;
    const unsigned grid = static_cast<unsigned>(blocks < 4096 ? blocks : 4096);
    k_nz_count<T><<<grid, 256, 0, s>>>(sv, N, eps, nchunks, counts);
    cuda_check(cudaGetLastError(), "k_nz_count launch");
    note_launch();
}
template <class T>
void launch_nz_select(cudaStream_t s, const cx<T> *sv, u64 N, T eps, const u64 *prefix, u64 nchunks, const u64 *rank,
                      u64 steps, u64 *tidx, T *tplog) {
    const u64 blocks = (steps + 7) / 8;
    const unsigned grid = static_cast<unsigned>(blocks < 4096 ? blocks : 4096);
    k_nz_select<T><<<grid, 256, 0, s>>>(sv, N, eps, prefix, nchunks, rank, steps, tidx, tplog);
    cuda_check(cudaGetLastError(), "k_nz_select launch");
    note_launch();
}
template <class T>
void launch_mcmc_chain_nz(cudaStream_t s, const cx<T> *sv, const u64 *tidx, const T *tplog, const T *ran, u64 steps,
                          u64 burnin, u64 *out) {
    k_mcmc_chain_nz<T><<<1, 256, 0, s>>>(sv, tidx, tplog, ran, steps, burnin, out);
    cuda_check(cudaGetLastError(), "k_mcmc_chain_nz launch");
    note_launch();
}
template <class T>
void launch_mcmc_chain_local(cudaStream_t s, const cx<T> *sv, const unsigned char *site, const unsigned char *value,
                             const T *ran, u64 steps, u64 burnin, u64 *out) {
    k_mcmc_chain_local<T><<<1, 32, 0, s>>>(sv, site, value, ran, steps, burnin, out);
    cuda_check(cudaGetLastError(), "k_mcmc_chain_local launch");
    note_launch();
}
void launch_index_bits(cudaStream_t s, const u64 *idx, u64 shots, int n, long long *out) {
    const u64 total = shots * static_cast<u64>(n);
    if (total == 0) {
        return;
    }
    k_index_bits<<<grid_for(total, 256, 8), 256, 0, s>>>(idx, shots, n, out);
    cuda_check(cudaGetLastError(), "k_index_bits launch");
    note_launch();
}

#define PLGB_MCMC_INST(T)                                                                                         \
    template void launch_nz_count<T>(cudaStream_t, const cx<T> *, u64, T, u64, unsigned *);                       \
    template void launch_nz_select<T>(cudaStream_t, const cx<T> *, u64, T, const u64 *, u64, const u64 *, u64,   \
                                      u64 *, T *);                                                                \
    template void launch_mcmc_chain_nz<T>(cudaStream_t, const cx<T> *, const u64 *, const T *, const T *, u64,   \
                                          u64, u64 *);                                                            \
    template void launch_mcmc_chain_local<T>(cudaStream_t, const cx<T> *, const unsigned char *,                 \
                                             const unsigned char *, const T *, u64, u64, u64 *);
PLGB_MCMC_INST(float)
PLGB_MCMC_INST(double)

} // namespace plgb
