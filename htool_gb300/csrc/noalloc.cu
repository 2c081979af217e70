// Product entry point that allocates nothing.
//
// The regular product (HMatrix::mvprod) keeps its working vectors -- the
// gathered input and the phase-1 partial sums -- in device buffers that it
// grows with cudaMalloc the first time a larger number of right-hand sides is
// requested.  Some callers cannot let a library allocate device memory at
// that point: a process whose framework has already reserved the GPU's
// memory for its own pool, or an iterative solver that drives the product
// from a hot loop where an allocation (and the device synchronisation it
// implies) is not acceptable.  This file gives them one product call whose
// working memory is a fixed array in the library's own device image.
// CUDA loads a module's device globals lazily, so the array is brought in
// by an explicit address lookup, done when an H-matrix is created on the
// device (noalloc_reserve): by the time a caller's pool has taken the GPU's
// memory, the array is already resident.
#include "hmatrix.hpp"

#include <mutex>

namespace htgpu {

// 16 MiB of working memory per device, held by every GPU on which an
// H-matrix was created (or an allocation-free product was called) until the
// process exits.  A product needs 2 * nb_cols * mu
// doubles for the gathered input and its float split, one slot for the
// input's exponent, (phase-1 partial-sum slots) * mu doubles and
// (per-cluster partial-sum rows) * mu doubles.
constexpr std::size_t kNoAllocScratchDoubles = 2u * 1024u * 1024u;
static __device__ __align__(256) double g_noalloc_scratch[kNoAllocScratchDoubles];

namespace {
constexpr int kMaxDevices = 64;
std::mutex g_scratch_mutex;
double *g_scratch_addr[kMaxDevices] = {nullptr};

// Device address of the array on `device` (the current device).  Looked up
// once per device; host code must not use the symbol itself, which is only
// a host-side stand-in for the device array.
double *scratch_on(int device) {
    if (device < 0 || device >= kMaxDevices)
        throw Error(1, "[Htool error] device index out of range for the allocation-free product");
    std::lock_guard<std::mutex> lock(g_scratch_mutex);
    if (!g_scratch_addr[device]) {
        void *p        = nullptr;
        cudaError_t rc = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (rc != cudaSuccess)
            throw Error(3, std::string("[Htool error] CUDA: cudaGetSymbolAddress of the allocation-free scratch failed: ") + cudaGetErrorString(rc));
        g_scratch_addr[device] = static_cast<double *>(p);
    }
    return g_scratch_addr[device];
}
} // namespace

void noalloc_reserve(int device) noexcept {
    try {
        scratch_on(device);
    } catch (...) {
        // leave the failure to the first allocation-free product, which
        // repeats the lookup and reports it; clear the non-sticky error so
        // that it does not surface in an unrelated call
        cudaGetLastError();
    }
}

std::size_t HMatrix::noalloc_scratch_need(int mu) const {
    // gathered input and its split, each rounded up to 32 doubles (256
    // bytes), 32 doubles for the exponent word, then the partial sums
    const std::size_t xp_len = ((std::size_t)nc * mu + 31) / 32 * 32;
    return 2 * xp_len + 32 + (std::size_t)std::max<long long>(a_slots, 1) * mu + (std::size_t)std::max<long long>(zlen_, 1) * mu;
}

void HMatrix::mvprod_noalloc(const double *in, double *out, int mu, cudaStream_t st) {
    // messages are only built on failure: the success path makes no host
    // allocation either
    if (mu < 1)
        throw Error(1, "[Htool error] number of right-hand sides must be positive");
    if (in == nullptr || out == nullptr)
        throw Error(1, "[Htool error] null input or output");
    const std::size_t need = noalloc_scratch_need(mu);
    if (need > kNoAllocScratchDoubles)
        throw Error(1, "[Htool error] the allocation-free product needs " + std::to_string(need) + " doubles of working memory for mu = " + std::to_string(mu) + ", more than its fixed " +
                           std::to_string(kNoAllocScratchDoubles) + "; use the regular product");
    HTGPU_CUDA(cudaSetDevice(device_));
    if (!st)
        st = stream_;
    double *base          = scratch_on(device_);
    const std::size_t xpl = ((std::size_t)nc * mu + 31) / 32 * 32;
    double *xpw           = base;
    F2 *xsw               = reinterpret_cast<F2 *>(base + xpl);
    int *xew              = reinterpret_cast<int *>(base + 2 * xpl);
    double *Aw            = base + 2 * xpl + 32;
    double *zw            = Aw + (std::size_t)std::max<long long>(a_slots, 1) * mu;
    // the exponent word is cleared by launch_xexp (an asynchronous memset,
    // no allocation); every other entry is written before it is read
    launch_product_with(in, out, mu, false, st, xpw, xsw, xew, Aw, zw);
}

} // namespace htgpu
