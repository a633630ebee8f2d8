// Allocation-free expectation value of a Hermitian matrix on at most five
// wires: the body of plgb_meas_expval_matrix_noalloc (include/pl_gb300.h).
//
// Why it exists.  plgb_meas_expval_matrix stages the matrix in the state
// vector's device scratch, which grows on demand: a larger matrix than any
// before frees the old buffer and calls cudaMalloc.  cudaFree waits for all
// work on the device, and cudaMalloc can fail once the device is full.  A
// caller that has filled the device with state vectors up to its memory
// budget (a serving loop admitting requests against a fixed number of GB),
// or one that runs measurements between latency-bound launches on other
// streams, cannot accept either inside a measurement.  This variant keeps
// its scratch in one fixed file-scope device array and allocates nothing.
//
// Limits and contract.
//  * At most kNoAllocMaxWires = 5 wires (a 32 x 32 matrix, 16 KiB of
//    complex128); larger requests are rejected with PLGB_ERR_INVALID.
//  * The first call on each device does the set-up: it resolves the
//    device address of the array with cudaGetSymbolAddress, with that device
//    current.
//  * Every call copies the matrix in from the host stack and synchronises
//    the state vector's stream before it returns, so no call may be made
//    while any stream is being captured.
//  * A lazy handle with gates still queued is rejected (PLGB_ERR_INVALID):
//    running the queue compiles and uploads a fused program, which
//    allocates.
//  * Nothing in the array needs to start at zero: the matrix is copied in
//    before each launch, every reduction block writes its own partial slot,
//    and the final reduction overwrites the result slot.
//  * The array is shared by every caller on a device.  Two calls that
//    overlap in time (from two host threads, or with another state vector on
//    another stream of the same device) race on it and can return wrong
//    values; serialise them.  A call returns only after its stream has
//    drained, so calls made one after another are safe.
#include "host.hpp"

#include <atomic>
#include <mutex>

namespace plgb {

namespace {

constexpr int kNoAllocMaxWires = 5;
constexpr int kNoAllocMaxDim = 1 << kNoAllocMaxWires;
constexpr int kNoAllocMaxDevices = 64;

struct NoAllocScratch {
    double mat[2 * kNoAllocMaxDim * kNoAllocMaxDim]; // the matrix as cx<T>, row-major
    double partials[kReduceBlocks];                  // one slot per reduction block
    double result[32];                               // final sum in result[0]
};

static __device__ __align__(256) NoAllocScratch g_noalloc_scratch;

std::atomic<NoAllocScratch *> g_scratch_ptr[kNoAllocMaxDevices];
std::mutex g_setup_mu;

// Device address of the array on `dev`, resolved once per device.
NoAllocScratch *scratch_on(int dev) {
    PLGB_REQUIRE(dev >= 0 && dev < kNoAllocMaxDevices, "device ordinal out of range for the no-allocation scratch");
    NoAllocScratch *p = g_scratch_ptr[dev].load(std::memory_order_acquire);
    if (p != nullptr) {
        return p;
    }
    std::lock_guard<std::mutex> lk(g_setup_mu);
    p = g_scratch_ptr[dev].load(std::memory_order_relaxed);
    if (p != nullptr) {
        return p;
    }
    int prev = -1;
    cuda_check(cudaGetDevice(&prev), "cudaGetDevice");
    if (prev != dev) {
        cuda_check(cudaSetDevice(dev), "cudaSetDevice");
    }
    void *addr = nullptr;
    const cudaError_t rc = cudaGetSymbolAddress(&addr, g_noalloc_scratch);
    if (prev != dev) {
        cuda_check(cudaSetDevice(prev), "cudaSetDevice");
    }
    cuda_check(rc, "cudaGetSymbolAddress(no-allocation scratch)");
    PLGB_REQUIRE(addr != nullptr, "cudaGetSymbolAddress returned a null address");
    p = static_cast<NoAllocScratch *>(addr);
    g_scratch_ptr[dev].store(p, std::memory_order_release);
    return p;
}

} // namespace

template <class T>
double expval_matrix_noalloc(StateVector<T> &sv, const double *matrix, const int64_t *wires, int nw) {
    // Same reduction as Measure<T>::expval_matrix for k <= 5 wires
    // (MeasurementsLQubit.hpp:213-238), with fixed scratch.
    PLGB_REQUIRE(nw >= 1, "Number of wires must be larger than 0");
    PLGB_REQUIRE(nw <= kNoAllocMaxWires,
                 "plgb_meas_expval_matrix_noalloc takes at most 5 wires (a 32 x 32 matrix); use "
                 "plgb_meas_expval_matrix for larger observables");
    const int k = nw;
    const int D = 1 << k;
    int tb[kNoAllocMaxWires];
    for (int i = 0; i < k; i++) {
        tb[i] = sv.bit_of(wires[i]);
        for (int j = 0; j < i; j++) {
            PLGB_REQUIRE(tb[j] != tb[i], "wires must be unique");
        }
    }
    GroupGeom g{};
    g.nins = k;
    for (int i = 0; i < k; i++) {
        g.ins[i] = tb[i];
    }
    for (int i = 1; i < k; i++) { // sort the inserted bits ascending
        for (int j = i; j > 0 && g.ins[j - 1] > g.ins[j]; j--) {
            const int t = g.ins[j];
            g.ins[j] = g.ins[j - 1];
            g.ins[j - 1] = t;
        }
    }
    g.ngroups = sv.length() >> k;
    LocalOffsets lo{};
    for (int j = 0; j < D; j++) {
        u64 o = 0;
        for (int m = 0; m < k; m++) {
            if ((j >> (k - 1 - m)) & 1) {
                o |= u64{1} << tb[m];
            }
        }
        lo.off[j] = o;
    }
    cx<T> mat[kNoAllocMaxDim * kNoAllocMaxDim];
    for (int i = 0; i < D * D; i++) {
        mat[i] = cx<T>{static_cast<T>(matrix[2 * i]), static_cast<T>(matrix[2 * i + 1])};
    }

    cudaPointerAttributes attr{};
    cuda_check(cudaPointerGetAttributes(&attr, sv.data()), "cudaPointerGetAttributes");
    NoAllocScratch *scr = scratch_on(attr.device);
    cx<T> *dmat = reinterpret_cast<cx<T> *>(scr->mat);
    const cudaStream_t s = sv.stream();
    cuda_check(cudaMemcpyAsync(dmat, mat, static_cast<size_t>(D) * D * sizeof(cx<T>), cudaMemcpyHostToDevice, s),
               "H2D");
    reduce_expval_matrix<T>(s, sv.data(), g, k, lo, dmat, scr->partials, scr->result);
    double out = 0.0;
    cuda_check(cudaMemcpyAsync(&out, scr->result, sizeof(double), cudaMemcpyDeviceToHost, s), "D2H");
    cuda_check(cudaStreamSynchronize(s), "cudaStreamSynchronize");
    return out;
}

template double expval_matrix_noalloc<float>(StateVector<float> &, const double *, const int64_t *, int);
template double expval_matrix_noalloc<double>(StateVector<double> &, const double *, const int64_t *, int);

} // namespace plgb
