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
// Per CTA (256 threads, one per SM): the three splits of A (32 KiB each)
// stay in shared memory for every tile.  Tiles arrive by 16-byte
// asynchronous copies (cp.async) into two raw buffers, two tiles ahead, so
// the loads of the next tiles overlap this tile's work.  Per tile the 4096
// amplitudes are split and written to the three B operands in the
// canonical no-swizzle K-major layout (8 x 16-byte core matrices), one
// thread issues the 48 MMAs and commits them to an mbarrier, all threads
// read D back from tensor memory (tcgen05.ld), stage the tile in shared
// memory in global order and store it coalesced.
//
// Tile geometry: the tile's 12 local bits are the six block bits and the
// six lowest other bits; local index jj enumerates them in ascending global
// position, so consecutive threads touch consecutive addresses.  The member
// index u (row of A in member order: bit q = the q-th lowest block bit) and
// group index g are bit permutations of jj.  The split reads the raw tile
// per (u, g) so that a warp writes 32 consecutive words of B; the raw
// buffer and the output stage are XOR-swizzled (TcGeom) so that those reads
// and the stage writes per tensor-memory lane are free of bank conflicts.
//
// Every wait is bounded: an mbarrier that does not complete within the
// limit sets the error word, and the CTA stops issuing, frees its tensor
// memory and returns; the host reads the word after the launch.
#include "kernels_tc.hpp"


#include <atomic>
#include <cstring>
#include <vector>

namespace plgb {

namespace {

// 256 threads (8 warps).  The index maps below also hold for 512 threads
// (kTcThreadBits = 9), which measured slower on a GB300 (0.61 against
// 0.54 ms for a 2^26-amplitude gate): the phases of a tile are separated by
// barriers, and more warps per phase do not shorten the chain.
constexpr int kTcThreadBits = 8;
constexpr int kTcThreads = 1 << kTcThreadBits;
constexpr int kTcWarps = kTcThreads / 32;
constexpr int kTcCols = 64 / (kTcWarps / 4);     // accumulator columns a warp reads back
constexpr int kTcTileBits = 12;                  // 4096 amplitudes per tile
constexpr int kTcPerThread = (1 << kTcTileBits) / kTcThreads; // amplitudes per thread and tile
constexpr unsigned kTcASplitBytes = 128u * 128u * 2u;         // one BF16 split of A: 32 KiB
constexpr unsigned kTcBSplitBytes = 64u * 128u * 2u;          // one split of B: 16 KiB
constexpr unsigned kTcRawBytes = 4096u * 8u;                 // one tile of complex64: 32 KiB
constexpr int kTcChunksPerThread = 4096 * 8 / 16 / kTcThreads; // 16-byte copies per thread and tile
constexpr unsigned kTcSmemBytes = 3 * kTcASplitBytes + 3 * kTcBSplitBytes + 2 * kTcRawBytes + 64;
constexpr unsigned kTcTmemCols = 64;             // the 128 x 64 FP32 accumulator
constexpr long long kTcWaitLimit = 1ll << 22;    // mbarrier polls before giving up
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

// 16 consecutive FP32 columns of this thread's tensor-memory lane
[[maybe_unused]] __device__ __forceinline__ void tc_ld(unsigned taddr, float (&v)[16]) {
    unsigned r[16];
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 "
                 "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, [%16];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
                   "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
                   "=r"(r[14]), "=r"(r[15])
                 : "r"(taddr)
                 : "memory");
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int c = 0; c < 16; c++) {
        v[c] = __uint_as_float(r[c]);
    }
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

__device__ __forceinline__ void cp_async16(unsigned dst, const void *src) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(dst), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait1() { asm volatile("cp.async.wait_group 1;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait0() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }

// the tile number deposited into the non-local bits
__device__ __forceinline__ u64 tile_base(const TcGeom &geom, u64 tile) {
    u64 base = 0;
    for (int q = 0; q < geom.nglob; q++) {
        base |= (tile & 1u) << geom.glob[q];
        tile >>= 1;
    }
    return base;
}

// Copy one tile (4096 amplitudes) into a raw buffer with 16-byte
// asynchronous copies: chunk c holds amplitudes 2c and 2c + 1 of the local
// order, adjacent in memory (local bit 0 is index bit 0), placed at their
// swizzled position.
__device__ __forceinline__ void fetch_tile(const float2 *sv, u64 base, const u64 *coff, const unsigned *cdst,
                                           unsigned raw) {
#pragma unroll
    for (int r = 0; r < kTcChunksPerThread; r++) {
        cp_async16(raw + cdst[r], sv + (base | coff[r]));
    }
}

__global__ void __launch_bounds__(kTcThreads, 1)
    k_dense6_tc(float2 *__restrict__ sv, TcGeom geom, const uint4 *__restrict__ a_img, int *__restrict__ err) {
    extern __shared__ __align__(1024) unsigned char smem[];
    // A splits h, m, l | B splits h, m, l | two raw tile buffers | mbarrier |
    // tensor-memory address
    unsigned char *A0 = smem;
    unsigned char *B0 = smem + 3 * kTcASplitBytes;
    unsigned char *R0 = B0 + 3 * kTcBSplitBytes;
    unsigned long long *mbar = reinterpret_cast<unsigned long long *>(R0 + 2 * kTcRawBytes);
    unsigned *tslot = reinterpret_cast<unsigned *>(R0 + 2 * kTcRawBytes + 16);
    float2 *stage = reinterpret_cast<float2 *>(B0); // the tile in local order, after the MMAs (32 of 48 KiB)

    const unsigned tid = threadIdx.x;
    const unsigned warp = tid >> 5, lane = tid & 31u;

    for (unsigned i = tid; i < 3 * kTcASplitBytes / 16; i += kTcThreads) {
        reinterpret_cast<uint4 *>(smem)[i] = a_img[i];
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tslot)),
                     "r"(kTcTmemCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (tid == 0) {
        mbar_init(smem_u32(mbar), 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    proxy_fence_smem(); // A written by the generic proxy, read by the MMAs
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const unsigned tmem = *tslot;

    // XOR swizzle of a local index (linear in its bits 4-11)
    auto swz = [&](unsigned jj, const unsigned short *h) {
        unsigned x = jj;
#pragma unroll
        for (int q = 4; q < 12; q++) {
            x ^= ((jj >> q) & 1u) ? h[q] : 0u;
        }
        return x;
    };
    // store phase: local index jj = r * kTcThreads + tid, read from the
    // swizzled stage, written to global memory (consecutive threads,
    // consecutive addresses)
    u64 off_t = 0;
    for (int q = 0; q < kTcThreadBits; q++) {
        off_t |= static_cast<u64>((tid >> q) & 1u) << geom.lbit[q];
    }
    const unsigned st_t = swz(tid, geom.hst);
    unsigned st_r[kTcPerThread];
    u64 off_r[kTcPerThread];
#pragma unroll
    for (int r = 0; r < kTcPerThread; r++) {
        st_r[r] = swz(static_cast<unsigned>(r) << kTcThreadBits, geom.hst);
        u64 o = 0;
        for (int q = 0; q < kTcTileBits - kTcThreadBits; q++) {
            o |= static_cast<u64>((r >> q) & 1) << geom.lbit[kTcThreadBits + q];
        }
        off_r[r] = o;
    }
    // split phase: this thread handles group g = (lane >> 2) | ((warp & 7)
    // << 3) and member u = (lane & 3) | (uh << 2), uh = (warp >> 3) | (r <<
    // (threads bits - 8)), so a warp's B stores are 32 consecutive words;
    // the raw tile is read at its swizzled position
    constexpr int kUs = kTcThreadBits - 8; // member bits from the warp index
    const unsigned g_me = (lane >> 2) | ((warp & 7u) << 3);
    const unsigned raw_t =
        swz(geom.jj_of_u[(lane & 3u) | ((warp >> 3) << 2)] | geom.jj_of_g[g_me], geom.hraw);
    unsigned raw_r[kTcPerThread];
#pragma unroll
    for (int r = 0; r < kTcPerThread; r++) {
        raw_r[r] = swz(geom.jj_of_u[static_cast<unsigned>(r) << (2 + kUs)], geom.hraw);
    }
    // kmajor_off(g, 2u) for r = 0
    const unsigned b_t = ((warp & 7u) * 16u + (warp >> 3)) * 128u + lane * 4u;
    // global offsets and swizzled raw positions of this thread's copy
    // chunks: local index 2c with c = r * 256 + tid
    u64 coff[kTcChunksPerThread];
    unsigned cdst[kTcChunksPerThread];
#pragma unroll
    for (int r = 0; r < kTcChunksPerThread; r++) {
        const unsigned c = static_cast<unsigned>(r) * kTcThreads + tid;
        u64 o = 0;
        for (int q = 0; q < 11; q++) {
            o |= static_cast<u64>((c >> q) & 1u) << geom.lbit[q + 1];
        }
        coff[r] = o;
        cdst[r] = swz(2u * c, geom.hraw) * 8u; // byte offset of the pair (bit 0 is never swizzled)
    }
    // stage writes: tensor-memory lane m = 32 (warp % 4) + lane is member
    // u = m / 2, component m % 2
    const unsigned row = 32u * (warp & 3u) + lane;
    const unsigned st_u = geom.st_of_u[row >> 1];
    const unsigned col0 = static_cast<unsigned>(kTcCols) * (warp >> 2);

    const unsigned a0 = smem_u32(A0), b0 = smem_u32(B0), r0 = smem_u32(R0);
    // the address field of a descriptor is 14 bits of bytes >> 4: every
    // operand address (below 228 KiB) fits, so offsets add without carry
    const unsigned long long adesc0 = smem_desc(a0, kLbo, kSbo), bdesc0 = smem_desc(b0, kLbo, kSbo);
    const unsigned bar = smem_u32(mbar);
    unsigned phase = 0;
    bool failed = false;

    // prefetch the first two tiles (one commit group each, empty when absent)
    const u64 stride = gridDim.x;
    u64 tile = blockIdx.x;
    for (int k = 0; k < 2; k++) {
        const u64 t = tile + static_cast<u64>(k) * stride;
        if (t < geom.ntiles) {
            fetch_tile(sv, tile_base(geom, t), coff, cdst, r0 + static_cast<unsigned>(k) * kTcRawBytes);
        }
        cp_async_commit();
    }
    for (unsigned buf = 0; tile < geom.ntiles && !failed; tile += stride, buf ^= 1u) {
        const u64 base = tile_base(geom, tile);
        cp_async_wait1(); // this tile's group has landed (the next one may be in flight)
        __syncthreads();
        // split the tile into the B operands
        const float2 *raw = reinterpret_cast<const float2 *>(R0 + buf * kTcRawBytes);
#pragma unroll
        for (int r = 0; r < kTcPerThread; r++) {
            const float2 v = raw[raw_t ^ raw_r[r]];
            const unsigned o = b_t + (static_cast<unsigned>(r) << kUs) * 128u; // (re, im) adjacent: k = 2u, 2u + 1
            unsigned h, m, l;
            split3x2(v.x, v.y, h, m, l);
            *reinterpret_cast<unsigned *>(B0 + o) = h;
            *reinterpret_cast<unsigned *>(B0 + kTcBSplitBytes + o) = m;
            *reinterpret_cast<unsigned *>(B0 + 2 * kTcBSplitBytes + o) = l;
        }
        proxy_fence_smem();
        tc_fence_before();
        __syncthreads();
        // the raw buffer is consumed: fetch the tile after next into it
        {
            const u64 t = tile + 2 * stride;
            if (t < geom.ntiles) {
                fetch_tile(sv, tile_base(geom, t), coff, cdst, r0 + buf * kTcRawBytes);
            }
            cp_async_commit();
        }
        if (tid == 0) {
            tc_fence_after();
            // split pairs (A, B), smallest products first: l.h, h.l, m.m, m.h,
            // h.m, h.h.  The 48 descriptors are the two base descriptors plus
            // compile-time offsets in the address field (bytes >> 4): a split
            // stride, and 256 bytes (two 16-byte core columns, K = 16) per step.
#pragma unroll
            for (int p = 0; p < 6; p++) {
#pragma unroll
                for (int ks = 0; ks < 8; ks++) {
                    const unsigned long long ad =
                        adesc0 + ((tc_pa(p) * kTcASplitBytes + static_cast<unsigned>(ks) * 256u) >> 4);
                    const unsigned long long bd =
                        bdesc0 + ((tc_pb(p) * kTcBSplitBytes + static_cast<unsigned>(ks) * 256u) >> 4);
                    tc_mma_bf16(tmem, ad, bd, (p | ks) != 0 ? 1u : 0u);
                }
            }
            tc_commit(bar);
        }
        // wait for the MMAs (bounded)
        long long polls = 0;
        while (!mbar_try_wait(bar, phase)) {
            if (++polls > kTcWaitLimit) {
                failed = true;
                break;
            }
        }
        failed = __syncthreads_or(failed) != 0;
        if (failed) {
            if (tid == 0) {
                atomicExch(err, 1);
            }
            break;
        }
        phase ^= 1u;
        tc_fence_after();
        // D row m = 32 (warp % 4) + lane; warp w reads kTcCols columns from
        // kTcCols * (w / 4).  The MMAs have consumed B, so the stage (over
        // the B splits) may be written.
        {
            float d[kTcCols];
            tc_ld(tmem + ((32u * (warp & 3u)) << 16) + col0, d);
            float *st = reinterpret_cast<float *>(stage);
            const unsigned comp = row & 1u;
#pragma unroll
            for (int c = 0; c < kTcCols; c++) {
                st[2u * (st_u ^ geom.st_of_g[col0 + static_cast<unsigned>(c)]) + comp] = d[c];
            }
        }
        tc_fence_before();
        __syncthreads();
#pragma unroll
        for (int r = 0; r < kTcPerThread; r++) {
            __stcs(&sv[base | off_t | off_r[r]], stage[st_t ^ st_r[r]]);
        }
        __syncthreads(); // the stage is read before the next tile's B writes
    }
    cp_async_wait0(); // no copy into shared memory outlives the CTA
    __syncthreads();
    if (warp == 0) {
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTcTmemCols)
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
    if (g.lbit[0] != 0) { // the 16-byte copies need adjacent amplitude pairs
        return false;
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
    // Swizzles: the jj bits that vary across the lanes of a half-warp at
    // positions 4 and up are mapped onto the free positions among the
    // bank-selecting ones.  Raw buffer (8-byte reads, pairs kept together):
    // lanes vary u0, u1, g0, g1; positions 1-3 are available.  Stage
    // (4-byte writes of (u, component)): lanes vary u0-u3; positions 0-3.
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
    const int raw_lanes[4] = {upos[0], upos[1], gpos[0], gpos[1]};
    const int st_lanes[4] = {upos[0], upos[1], upos[2], upos[3]};
    assign(raw_lanes, 4, 1, g.hraw);
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
        cuda_check(cudaFuncSetAttribute(k_dense6_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, kTcSmemBytes),
                   "cudaFuncSetAttribute(k_dense6_tc)");
        attr_set = true;
    }
    const u64 want = geom.ntiles;
    const u64 cap = static_cast<u64>(LaunchGeom::sm_count());
    const unsigned grid = static_cast<unsigned>(want < cap ? want : cap);
    k_dense6_tc<<<grid, kTcThreads, kTcSmemBytes, s>>>(reinterpret_cast<float2 *>(sv), geom,
                                                        reinterpret_cast<const uint4 *>(a_img), err);
    cuda_check(cudaGetLastError(), "k_dense6_tc launch");
    note_launch();
}

} // namespace plgb
