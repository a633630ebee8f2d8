// Dense 6-wire blocks of complex64 gates on the 5th-generation tensor cores.
//
// A dense 64 x 64 complex matrix U on six target bits maps every group of 64
// amplitudes (the indices that differ only in those bits) to U times the
// group.  Over a tile of 64 groups that is one real GEMM:
//     D[128 x 64] = A[128 x 128] . B[128 x 64]
// with A the real form of U (rows 2r + out-component, columns 2c +
// in-component: [[Ur, -Ui], [Ui, Ur]] interleaved) and B the tile's groups
// (column n = group, row 2c + component).  It runs as tcgen05.mma with
// kind::f16 on BF16 operands (M = 128, N = 64, K = 16 per instruction), the
// FP32 accumulator in tensor memory.  BF16 keeps 8 significant bits, so
// every FP32 operand is split into three: x = h + m + l, h = bf16(x),
// m = bf16(x - h), l = bf16(x - h - m), each rounded to nearest, which
// represents the 24-bit significand exactly.  D is the sum of the six
// products whose split indices add up to at most 2 (l.h, h.l, m.m, m.h,
// h.m, h.h, smallest first); the three omitted ones are below 2^-24 of the
// result, so a block is as accurate as an FP32 matrix product.
//
// Per CTA (one per SM, warp-specialized, see k_dense6_tc): the three splits
// of A (32 KiB each) stay in shared memory for every tile; B (three splits,
// canonical no-swizzle K-major layout of 8 x 16-byte core matrices) and the
// tensor-memory accumulator are double-buffered, so the split of one tile,
// the MMAs of the next and the read-back and store of the previous one run
// at the same time.
//
// Tile geometry: the tile's 12 local bits are the six block bits and the
// six lowest other bits; local index jj enumerates them in ascending global
// position.  The member index u (row of A in member order: bit q = the q-th
// lowest block bit) and group index g are bit permutations of jj.  The split
// threads read the amplitudes of (u, g) straight from global memory (in
// whole 32-byte sectors: a warp covers two or three of the lowest index
// bits) so that a warp writes 32 consecutive words of B; the output stage is
// XOR-swizzled (TcGeom) so that the writes per tensor-memory lane are free of
// bank conflicts, and its reads in global order give coalesced stores.
//
// Every wait is bounded: an mbarrier that does not complete within the
// limit sets the error word and the CTA's abort flag; every role then
// leaves its loop, the MMA thread waits for the MMAs it issued, and the
// tensor memory is freed; the host reads the word after the launch.
#include "kernels_tc.hpp"


#include <atomic>
#include <cstring>
#include <string>
#include <vector>

namespace plgb {

namespace {

constexpr int kTcTileBits = 12;                          // 4096 amplitudes per tile
constexpr unsigned kTcASplitBytes = 128u * 128u * 2u;   // one BF16 split of A: 32 KiB
constexpr unsigned kTcBSplitBytes = 64u * 128u * 2u;    // one split of B: 16 KiB
constexpr long long kTcWaitLimit = 1ll << 22;           // mbarrier polls before giving up
// split of A and of B in each of the six products (0 = h, 1 = m, 2 = l)
__host__ __device__ constexpr unsigned tc_pa(int p) { return p == 0 ? 2u : (p == 2 || p == 3) ? 1u : 0u; }
__host__ __device__ constexpr unsigned tc_pb(int p) { return p == 1 ? 2u : (p == 2 || p == 4) ? 1u : 0u; }
static_assert(tc_pa(0) == 2 && tc_pb(0) == 0 && tc_pa(1) == 0 && tc_pb(1) == 2 && tc_pa(2) == 1 && tc_pb(2) == 1 &&
                  tc_pa(3) == 1 && tc_pb(3) == 0 && tc_pa(4) == 0 && tc_pb(4) == 1 && tc_pa(5) == 0 && tc_pb(5) == 0,
              "products l.h, h.l, m.m, m.h, h.m, h.h");

// byte offset of element (row, k) in a no-swizzle K-major operand with 128
// K elements of 2 bytes: core matrix (row / 8, k / 8) of 8 rows x 16 bytes;
// K-adjacent core matrices 128 B apart (LBO), 8-row groups 2048 B apart (SBO)
__host__ __device__ constexpr unsigned kmajor_off(unsigned row, unsigned k) {
    return ((row >> 3) * 16u + (k >> 3)) * 128u + (row & 7u) * 16u + (k & 7u) * 2u;
}
constexpr unsigned kLbo = 128u, kSbo = 2048u;

__device__ __forceinline__ unsigned smem_u32(const void *p) {
    return static_cast<unsigned>(__cvta_generic_to_shared(p));
}

// Shared-memory matrix descriptor (tcgen05): start address, leading
// (K-direction) and stride (M/N-direction) byte offsets, all >> 4; bits
// 46-47 = 1 (descriptor version); layout type 0 = no swizzle.
__device__ __forceinline__ unsigned long long smem_desc(unsigned addr, unsigned lbo, unsigned sbo) {
    unsigned long long d = 0;
    d |= static_cast<unsigned long long>((addr >> 4) & 0x3FFFu);
    d |= static_cast<unsigned long long>((lbo >> 4) & 0x3FFFu) << 16;
    d |= static_cast<unsigned long long>((sbo >> 4) & 0x3FFFu) << 32;
    d |= 1ull << 46;
    return d;
}

// Instruction descriptor, kind::f16: D in FP32 (bits 4-5 = 1), A and B
// BF16 (bits 7-9 and 10-12 = 1), both K-major, N >> 3 at bits 17-22,
// M >> 4 at bits 24-28.
constexpr unsigned kIdescBf16 = (1u << 4) | (1u << 7) | (1u << 10) | ((64u >> 3) << 17) | ((128u >> 4) << 24);

__device__ __forceinline__ void mbar_init(unsigned bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
// true once the barrier's phase with parity `phase` has completed
__device__ __forceinline__ bool mbar_try_wait(unsigned bar, unsigned phase) {
    unsigned ok = 0;
    asm volatile("{\n\t.reg .pred p;\n\t"
                 "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                 "selp.u32 %0, 1, 0, p;\n\t}"
                 : "=r"(ok)
                 : "r"(bar), "r"(phase)
                 : "memory");
    return ok != 0;
}

__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void proxy_fence_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__device__ __forceinline__ void tc_mma_bf16(unsigned dtmem, unsigned long long adesc, unsigned long long bdesc,
                                            unsigned accumulate) {
    asm volatile("{\n\t.reg .pred p;\n\t"
                 "setp.ne.u32 p, %4, 0;\n\t"
                 "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(dtmem),
                 "l"(adesc), "l"(bdesc), "r"(kIdescBf16), "r"(accumulate)
                 : "memory");
}
__device__ __forceinline__ void tc_commit(unsigned bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar)
                 : "memory");
}

// 32 consecutive FP32 columns of this thread's tensor-memory lane
__device__ __forceinline__ void tc_ld(unsigned taddr, float (&v)[32]) {
    unsigned r[32];
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x32.b32 "
                 "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, "
                 "%16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
                   "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
                   "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]),
                   "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]),
                   "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
                 : "r"(taddr)
                 : "memory");
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int c = 0; c < 32; c++) {
        v[c] = __uint_as_float(r[c]);
    }
}

// x = h + m + l for the two floats x, y at once: three BF16 values each,
// rounded to nearest (exact for FP32 inputs), returned as packed pairs
// (x in the low half, y in the high half: a B-operand word (re, im))
__device__ __forceinline__ void split3x2(float x, float y, unsigned &h, unsigned &m, unsigned &l) {
    asm("cvt.rn.bf16x2.f32 %0, %1, %2;" : "=r"(h) : "f"(y), "f"(x));
    const float rx = __fsub_rn(x, __uint_as_float(h << 16)), ry = __fsub_rn(y, __uint_as_float(h & 0xffff0000u));
    asm("cvt.rn.bf16x2.f32 %0, %1, %2;" : "=r"(m) : "f"(ry), "f"(rx));
    const float sx = __fsub_rn(rx, __uint_as_float(m << 16)), sy = __fsub_rn(ry, __uint_as_float(m & 0xffff0000u));
    asm("cvt.rn.bf16x2.f32 %0, %1, %2;" : "=r"(l) : "f"(sy), "f"(sx));
}


// the tile number deposited into the non-local bits
__device__ __forceinline__ u64 tile_base(const TcGeom &geom, u64 tile) {
    u64 base = 0;
    for (int q = 0; q < geom.nglob; q++) {
        base |= (tile & 1u) << geom.glob[q];
        tile >>= 1;
    }
    return base;
}

// Warp roles (544 threads, one CTA per SM):
//   split warps 0-7: load a tile's amplitudes straight from global memory
//     (the next tile's loads are in flight in registers while the current
//     one is split), split them into the B operand of buffer t % 2;
//   warp 16, one elected thread: issues the 48 MMAs of tile t into tensor
//     memory columns 64 (t % 2) .. + 63 and commits them to an mbarrier;
//   epilogue warps 8-15 (two per tensor-memory lane quarter, 32 columns
//     each): read tile t's accumulator, stage it in shared memory over B of
//     buffer t % 2 (its MMAs are complete) and store it coalesced.
// B and the accumulator are double-buffered, so the split of tile t + 1, the
// MMAs of tile t and the epilogue of tile t - 1 overlap.  Every hand-off is
// an mbarrier (B full, MMAs done, accumulator free, B free, stage written);
// every wait is bounded, and a wait that runs out sets the CTA's abort flag
// and the error word: all roles then leave their loops, the MMA thread waits
// (bounded) for the MMAs it issued, and tensor memory is freed.
constexpr int kWsSplitThreads = 256;
constexpr int kWsEpiThreads = 256;
constexpr int kWsThreads = kWsSplitThreads + kWsEpiThreads + 32;
constexpr int kWsRows = 4096 / kWsSplitThreads; // amplitudes per split / epilogue thread and tile (16)
constexpr unsigned kWsBBytes = 3 * kTcBSplitBytes;  // one B buffer (three splits): 48 KiB
constexpr unsigned kWsTmemCols = 128;               // two 128 x 64 FP32 accumulators
enum WsBar { kBFull = 0, kMDone = 2, kTFree = 4, kBFree = 6, kEStage = 8, kNumWsBars = 9 };
constexpr unsigned kWsTableBytes = 16;
constexpr unsigned kWsSmemBytes = 3 * kTcASplitBytes + 2 * kWsBBytes + kWsTableBytes + kNumWsBars * 8 + 32;

// bounded wait for the phase of `bar` with parity `phase`; false when the
// CTA aborted or the wait ran out (which aborts the CTA)
__device__ __forceinline__ bool ws_wait(unsigned bar, unsigned phase, volatile int *abort_flag, int *err) {
    long long polls = 0;
    while (!mbar_try_wait(bar, phase)) {
        if (*abort_flag) {
            return false;
        }
        if (++polls > kTcWaitLimit) {
            *abort_flag = 1;
            atomicExch(err, 1);
            return false;
        }
    }
    return true;
}
__device__ __forceinline__ void mbar_arrive(unsigned bar) {
    asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.shared::cta.b64 st, [%0];\n\t}" ::"r"(bar) : "memory");
}

__global__ void __launch_bounds__(kWsThreads, 1)
    k_dense6_tc(float2 *__restrict__ sv, TcGeom geom, const uint4 *__restrict__ a_img, int *__restrict__ err) {
    extern __shared__ __align__(1024) unsigned char smem[];
    // A splits h, m, l | B buffers 0, 1 (each splits h, m, l) | offset tables
    // | mbarriers | tensor-memory address | abort flag
    unsigned char *A0 = smem;
    unsigned char *Bbuf = smem + 3 * kTcASplitBytes;
    unsigned long long *bars = reinterpret_cast<unsigned long long *>(Bbuf + 2 * kWsBBytes + kWsTableBytes);
    unsigned *tslot = reinterpret_cast<unsigned *>(bars + kNumWsBars);
    volatile int *abort_flag = reinterpret_cast<volatile int *>(tslot + 1);

    const unsigned tid = threadIdx.x;
    const unsigned warp = tid >> 5, lane = tid & 31u;
    auto dep = [&](unsigned jj) { // local index -> offset of its bits in the full index
        u64 o = 0;
        for (int q = 0; q < kTcTileBits; q++) {
            o |= static_cast<u64>((jj >> q) & 1u) << geom.lbit[q];
        }
        return o;
    };
    auto swz = [&](unsigned jj) { // stage position of a local index
        unsigned x = jj;
#pragma unroll
        for (int q = 4; q < 12; q++) {
            x ^= ((jj >> q) & 1u) ? geom.hst[q] : 0u;
        }
        return x;
    };

    for (unsigned i = tid; i < 3 * kTcASplitBytes / 16; i += kWsThreads) {
        reinterpret_cast<uint4 *>(smem)[i] = a_img[i];
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tslot)),
                     "r"(kWsTmemCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (tid == 0) {
        for (int b = 0; b < 2; b++) {
            mbar_init(smem_u32(&bars[kBFull + b]), kWsSplitThreads);
            mbar_init(smem_u32(&bars[kMDone + b]), 1);
            mbar_init(smem_u32(&bars[kTFree + b]), kWsEpiThreads);
            mbar_init(smem_u32(&bars[kBFree + b]), kWsEpiThreads);
        }
        mbar_init(smem_u32(&bars[kEStage]), kWsEpiThreads);
        *abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    proxy_fence_smem(); // A written by the generic proxy, read by the MMAs
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const unsigned tmem = *tslot;
    const u64 stride = gridDim.x;

    if (warp < kWsSplitThreads / 32) {
        // ---------------------------------------------------------------- split
        // thread (warp w, lane l) row r: group g = (l >> 2) | (w << 3),
        // member u = (l & 3) | (r << 2)
        const unsigned g0 = (lane >> 2) | (warp << 3);
        const u64 off_t = dep(geom.jj_of_u[lane & 3u] | geom.jj_of_g[g0]);
        const unsigned b_t = (warp * 16u) * 128u + lane * 4u; // kmajor_off(g, 2 (lane & 3)); row r adds r * 128
        float2 cur[kWsRows], nxt[kWsRows];
        auto load = [&](float2 (&dst)[kWsRows], u64 tt) {
            const u64 base = tile_base(geom, tt) | off_t;
#pragma unroll
            for (int r = 0; r < kWsRows; r++) {
                dst[r] = __ldcs(&sv[base | geom.split_row_off[r]]);
            }
        };
        u64 tile = blockIdx.x;
        if (tile < geom.ntiles) {
            load(cur, tile);
        }
        auto step = [&](float2 (&now)[kWsRows], float2 (&next)[kWsRows], unsigned t) -> bool {
            const unsigned b = t & 1u, k = t >> 1;
            if (tile + stride < geom.ntiles) {
                load(next, tile + stride);
            }
            if (t >= 2 && !ws_wait(smem_u32(&bars[kBFree + b]), (k - 1) & 1u, abort_flag, err)) {
                return false;
            }
            unsigned char *B0 = Bbuf + b * kWsBBytes;
#pragma unroll
            for (int r = 0; r < kWsRows; r++) {
                // (re, im) adjacent: k = 2u, 2u + 1 of group g
                const unsigned o = b_t + static_cast<unsigned>(r) * 128u;
                unsigned h, m, l;
                split3x2(now[r].x, now[r].y, h, m, l);
                *reinterpret_cast<unsigned *>(B0 + o) = h;
                *reinterpret_cast<unsigned *>(B0 + kTcBSplitBytes + o) = m;
                *reinterpret_cast<unsigned *>(B0 + 2 * kTcBSplitBytes + o) = l;
            }
            proxy_fence_smem();
            mbar_arrive(smem_u32(&bars[kBFull + b]));
            return true;
        };
        for (unsigned t = 0; tile < geom.ntiles && !*abort_flag; t += 2) {
            if (!step(cur, nxt, t)) {
                break;
            }
            tile += stride;
            if (tile >= geom.ntiles || *abort_flag) {
                break;
            }
            if (!step(nxt, cur, t + 1)) {
                break;
            }
            tile += stride;
        }
    } else if (warp < (kWsSplitThreads + kWsEpiThreads) / 32) {
        // ------------------------------------------------------------- epilogue
        // two warps per tensor-memory lane quarter (warp % 4), each reading
        // 32 of the 64 accumulator columns
        const unsigned ew = warp % 4u, half = (warp - kWsSplitThreads / 32) / 4u, e = tid - kWsSplitThreads;
        const unsigned row = 32u * ew + lane; // accumulator row m: member m / 2, component m % 2
        const unsigned st_u = geom.st_of_u[row >> 1], comp = row & 1u;
        const u64 off_e = dep(e);
        const unsigned st_e = swz(e);
        unsigned t = 0;
        for (u64 tile = blockIdx.x; tile < geom.ntiles && !*abort_flag; tile += stride, t++) {
            const unsigned b = t & 1u, k = t >> 1;
            if (!ws_wait(smem_u32(&bars[kMDone + b]), k & 1u, abort_flag, err)) {
                break;
            }
            tc_fence_after();
            float d0[32];
            tc_ld(tmem + ((32u * ew) << 16) + 64u * b + 32u * half, d0);
            tc_fence_before();
            mbar_arrive(smem_u32(&bars[kTFree + b])); // the accumulator may be overwritten
            // stage over B of this buffer (its MMAs are complete)
            float *st = reinterpret_cast<float *>(Bbuf + b * kWsBBytes);
#pragma unroll
            for (int c = 0; c < 32; c++) {
                st[2u * (st_u ^ geom.st_of_g[32u * half + c]) + comp] = d0[c];
            }
            mbar_arrive(smem_u32(&bars[kEStage]));
            if (!ws_wait(smem_u32(&bars[kEStage]), t & 1u, abort_flag, err)) {
                break;
            }
            const float2 *stage = reinterpret_cast<const float2 *>(st);
            const u64 base = tile_base(geom, tile) | off_e;
#pragma unroll
            for (int r = 0; r < kWsRows; r++) {
                __stcs(&sv[base | geom.epi_row_off[r]], stage[st_e ^ geom.epi_row_st[r]]);
            }
            mbar_arrive(smem_u32(&bars[kBFree + b])); // the stage has been read
        }
    } else if (lane == 0) {
        // ------------------------------------------------------------------ MMA
        const unsigned a0 = smem_u32(A0);
        const unsigned long long adesc0 = smem_desc(a0, kLbo, kSbo);
        unsigned t = 0;
        bool issued = false;
        unsigned last_b = 0, last_k = 0;
        for (u64 tile = blockIdx.x; tile < geom.ntiles && !*abort_flag; tile += stride, t++) {
            const unsigned b = t & 1u, k = t >> 1;
            if (t >= 2 && !ws_wait(smem_u32(&bars[kTFree + b]), (k - 1) & 1u, abort_flag, err)) {
                break;
            }
            if (!ws_wait(smem_u32(&bars[kBFull + b]), k & 1u, abort_flag, err)) {
                break;
            }
            tc_fence_after();
            const unsigned long long bdesc0 = smem_desc(smem_u32(Bbuf + b * kWsBBytes), kLbo, kSbo);
#pragma unroll
            for (int p = 0; p < 6; p++) {
#pragma unroll
                for (int ks = 0; ks < 8; ks++) {
                    const unsigned long long ad =
                        adesc0 + ((tc_pa(p) * kTcASplitBytes + static_cast<unsigned>(ks) * 256u) >> 4);
                    const unsigned long long bd =
                        bdesc0 + ((tc_pb(p) * kTcBSplitBytes + static_cast<unsigned>(ks) * 256u) >> 4);
                    tc_mma_bf16(tmem + 64u * b, ad, bd, (p | ks) != 0 ? 1u : 0u);
                }
            }
            tc_commit(smem_u32(&bars[kMDone + b]));
            issued = true;
            last_b = b;
            last_k = k;
        }
        // no MMA may be in flight when the tensor memory is freed
        if (issued) {
            long long polls = 0;
            while (!mbar_try_wait(smem_u32(&bars[kMDone + last_b]), last_k & 1u) && ++polls <= kTcWaitLimit) {
            }
        }
    }
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kWsTmemCols)
                     : "memory");
    }
}

} // namespace

bool tc_geom_for(int n, const int *bits6, TcGeom &g) {
    if (n < kTcTileBits) {
        return false;
    }
    bool blk[64] = {};
    for (int m = 0; m < 6; m++) {
        if (bits6[m] < 0 || bits6[m] >= n || blk[bits6[m]]) {
            return false;
        }
        blk[bits6[m]] = true;
    }
    // local bits: the block bits and the six lowest others, ascending
    int bsel[6], gsel[6], nb = 0, ng = 0;
    for (int b = 0; b < n; b++) {
        if (blk[b]) {
            bsel[nb++] = b;
        } else if (ng < 6) {
            gsel[ng++] = b;
        }
    }
    bool loc[64] = {};
    for (int m = 0; m < 6; m++) {
        loc[bsel[m]] = true;
        loc[gsel[m]] = true;
    }
    std::memset(&g, 0, sizeof(g));
    int pos[64];
    int nl = 0;
    for (int b = 0; b < n; b++) {
        if (loc[b]) {
            pos[b] = nl;
            g.lbit[nl++] = b;
        } else {
            g.glob[g.nglob++] = b;
        }
    }
    g.ntiles = u64{1} << (n - kTcTileBits);
    int upos[6], gpos[6];
    for (int q = 0; q < 6; q++) {
        upos[q] = pos[bsel[q]];
        gpos[q] = pos[gsel[q]];
    }
    for (unsigned v = 0; v < 64; v++) {
        unsigned ju = 0, jg = 0, mi = 0;
        for (int q = 0; q < 6; q++) {
            if ((v >> q) & 1u) {
                ju |= 1u << upos[q];
                jg |= 1u << gpos[q];
                for (int m = 0; m < 6; m++) {
                    if (bits6[m] == bsel[q]) {
                        mi |= 1u << (5 - m); // bits6[0] = the matrix's most significant bit
                    }
                }
            }
        }
        g.jj_of_u[v] = static_cast<unsigned short>(ju);
        g.jj_of_g[v] = static_cast<unsigned short>(jg);
        g.mat_of_u[v] = static_cast<unsigned short>(mi);
    }
    // Stage swizzle: the jj bits that vary across the lanes of a warp's
    // 4-byte writes of (u, component) -- u0-u3 -- at positions 4 and up are
    // mapped onto the free positions among the bank-selecting ones 0-3.
    auto assign = [&](const int *lanes, int nlanes, int first, unsigned short *h) {
        bool used[4] = {};
        for (int i = 0; i < nlanes; i++) {
            if (lanes[i] >= first && lanes[i] < 4) {
                used[lanes[i]] = true;
            }
        }
        for (int i = 0; i < nlanes; i++) {
            if (lanes[i] < 4) {
                continue;
            }
            for (int s = first; s < 4; s++) {
                if (!used[s]) {
                    used[s] = true;
                    h[lanes[i]] = static_cast<unsigned short>(1u << s);
                    break;
                }
            }
        }
    };
    const int st_lanes[4] = {upos[0], upos[1], upos[2], upos[3]};
    assign(st_lanes, 4, 0, g.hst);
    auto swz = [&](unsigned jj, const unsigned short *h) {
        unsigned x = jj;
        for (int q = 4; q < 12; q++) {
            if ((jj >> q) & 1u) {
                x ^= h[q];
            }
        }
        return x;
    };
    for (unsigned v = 0; v < 64; v++) {
        g.st_of_u[v] = static_cast<unsigned short>(swz(g.jj_of_u[v], g.hst));
        g.st_of_g[v] = static_cast<unsigned short>(swz(g.jj_of_g[v], g.hst));
    }
    auto dep = [&](unsigned jj) {
        u64 o = 0;
        for (int q = 0; q < kTcTileBits; q++) {
            o |= static_cast<u64>((jj >> q) & 1u) << g.lbit[q];
        }
        return o;
    };
    for (unsigned r = 0; r < 16; r++) {
        g.split_row_off[r] = dep(g.jj_of_u[r << 2]);
        g.epi_row_off[r] = dep(r << 8);
        g.epi_row_st[r] = static_cast<unsigned short>(swz(r << 8, g.hst));
    }
    return true;
}

namespace {
// FP32 -> BF16 bits, rounded to nearest even (finite inputs)
unsigned short bf16_rn_bits(float x) {
    unsigned u;
    std::memcpy(&u, &x, 4);
    u += 0x7FFFu + ((u >> 16) & 1u);
    return static_cast<unsigned short>(u >> 16);
}
float bf16_to_float(unsigned short b) {
    const unsigned u = static_cast<unsigned>(b) << 16;
    float x;
    std::memcpy(&x, &u, 4);
    return x;
}
} // namespace

void tc_build_a_image(const cx<float> *U, const TcGeom &geom, unsigned short *img) {
    for (int m = 0; m < 128; m++) {
        for (int k = 0; k < 128; k++) {
            const int r = geom.mat_of_u[m >> 1], c = geom.mat_of_u[k >> 1];
            const cx<float> u = U[r * 64 + c];
            float v;
            if ((m & 1) == 0) {
                v = (k & 1) == 0 ? u.x : -u.y; // Re out = Ur Re in - Ui Im in
            } else {
                v = (k & 1) == 0 ? u.y : u.x;  // Im out = Ui Re in + Ur Im in
            }
            const unsigned short h = bf16_rn_bits(v);
            const float r1 = v - bf16_to_float(h);
            const unsigned short mm = bf16_rn_bits(r1);
            const float r2 = r1 - bf16_to_float(mm);
            const unsigned short l = bf16_rn_bits(r2);
            const unsigned o = kmajor_off(static_cast<unsigned>(m), static_cast<unsigned>(k)) / 2u;
            img[o] = h;
            img[kTcASplitBytes / 2u + o] = mm;
            img[kTcASplitBytes + o] = l;
        }
    }
}

size_t tc_a_image_bytes() { return 3 * kTcASplitBytes; }

namespace {
std::atomic<bool> g_tc_dense{true};
}
bool tc_dense_enabled() { return g_tc_dense.load(); }
bool set_tc_dense_enabled(bool on) { return g_tc_dense.exchange(on); }

void launch_dense6_tc(cudaStream_t s, cx<float> *sv, const TcGeom &geom, const unsigned short *a_img, int *err) {
    static bool attr_set = false;
    if (!attr_set) {
        cuda_check(cudaFuncSetAttribute(k_dense6_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, kWsSmemBytes),
                   "cudaFuncSetAttribute(k_dense6_tc)");
        attr_set = true;
    }
    const u64 want = geom.ntiles;
    const u64 cap = static_cast<u64>(LaunchGeom::sm_count());
    const unsigned grid = static_cast<unsigned>(want < cap ? want : cap);
    k_dense6_tc<<<grid, kWsThreads, kWsSmemBytes, s>>>(reinterpret_cast<float2 *>(sv), geom,
                                                       reinterpret_cast<const uint4 *>(a_img), err);
    const cudaError_t le = cudaGetLastError();
    if (le != cudaSuccess) {
        cudaFuncAttributes fa{};
        cudaFuncGetAttributes(&fa, k_dense6_tc);
        cuda_check(le, ("k_dense6_tc launch (" + std::to_string(kWsThreads) + " threads, " +
                        std::to_string(fa.numRegs) + " registers, max " + std::to_string(fa.maxThreadsPerBlock) +
                        " threads per block, " + std::to_string(kWsSmemBytes) + " B dynamic shared memory)")
                           .c_str());
    }
    note_launch();
}

} // namespace plgb
