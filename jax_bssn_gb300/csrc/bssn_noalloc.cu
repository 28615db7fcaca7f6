// bssn_rhs_noalloc: the BSSN right-hand side for callers that cannot
// allocate device memory.
//
// Some callers of this library are not allowed to call cudaMalloc: a host
// framework that owns every byte of device memory and forbids plug-ins from
// allocating, a long-running solver whose memory budget is fixed at start-up,
// or a loop that must not pay for the implicit synchronisation a
// cudaMalloc/cudaFree can bring.  bssn_rhs needs a work buffer that such a
// caller cannot provide on demand, so this entry point brings its own: a
// fixed-size array in device global memory that is part of the loaded
// library.
//
// The array is allocated by the CUDA driver when the library's device code is
// loaded on a GPU and stays allocated on every GPU that loaded it until the
// process exits.  Its size is stated below; arrays whose padded extent does
// not fit are rejected.  Nothing here calls cudaMalloc, cudaFree or an
// allocating library routine.
#include <cstddef>
#include <mutex>

#include <cuda_runtime.h>

#include "../../include/bssn_gb300.h"
#include "bssn_driver.h"

namespace {

// Largest array served: (nx+8)*(ny+8)*(nz+8) <= 21952 samples, e.g. 20x20x20.
constexpr size_t kMaxPaddedSamples = 21952;
// Work blocks bssn_rhs uses in its larger (kappa != 0) form: the padded
// state and RHS (21 each) and the RHS scratch (81 first-derivative blocks,
// 24 derived-field blocks and 6 damping-term blocks), from the same
// constants bssn_workspace_bytes uses.
constexpr size_t kBlocks = 2 * bssn::NCOMP + bssn::rhs_work_blocks(true);
static_assert(kBlocks == 153, "the stated size of the array (26.9 MB) assumes 153 blocks");
constexpr size_t kScratchValues = kBlocks * kMaxPaddedSamples;  // 26.9 MB of float64

// One array shared by every call on a device.  The address cache below is
// keyed by device index and assumes the device's primary context (the one the
// CUDA runtime uses); after cudaDeviceReset, or under a caller's own driver
// context, the cached address would be stale.  Host code must not pass the
// name of this array to a kernel: on the host it only stands in for the
// device symbol; its device address comes from cudaGetSymbolAddress.
static __device__ __align__(256) double g_rhs_scratch[kScratchValues];

constexpr int kMaxDevices = 64;
std::mutex g_mutex;
double* g_scratch_address[kMaxDevices] = {};

}  // namespace

extern "C" int bssn_rhs_noalloc(const BssnFields* in, BssnFields* out, const int32_t shape[3],
                                const BssnParams* params, void* stream) {
    if (shape == nullptr) return bssn::fail(BSSN_ERR_INVALID, "shape is null");
    const size_t need = bssn_workspace_bytes(BSSN_OP_RHS, shape, params);
    if (need == 0) return bssn::fail(BSSN_ERR_INVALID, "array extents must be positive");
    size_t padded = 1;
    for (int d = 0; d < 3; ++d) padded *= (size_t)shape[d] + 8;
    if (padded > kMaxPaddedSamples || need > sizeof(double) * kScratchValues)
        return bssn::fail(BSSN_ERR_INVALID,
                          "array too large for bssn_rhs_noalloc: (nx+8)*(ny+8)*(nz+8) must not exceed 21952 "
                          "samples (e.g. 20x20x20); use bssn_rhs with a caller-provided workspace");
    int device = 0;
    cudaError_t e = cudaGetDevice(&device);
    if (e != cudaSuccess) return bssn::cuda_status(e, "bssn_rhs_noalloc: cudaGetDevice");
    if (device < 0 || device >= kMaxDevices) return bssn::fail(BSSN_ERR_INVALID, "device index out of range");
    double* scratch = nullptr;
    {
        // First call on each device: look up the device address of the
        // array with that device current, once.
        std::lock_guard<std::mutex> lock(g_mutex);
        if (g_scratch_address[device] == nullptr) {
            void* address = nullptr;
            e = cudaGetSymbolAddress(&address, g_rhs_scratch);
            if (e != cudaSuccess) return bssn::cuda_status(e, "bssn_rhs_noalloc: cudaGetSymbolAddress");
            g_scratch_address[device] = static_cast<double*>(address);
        }
        scratch = g_scratch_address[device];
    }
    // Every scratch value the RHS kernels read is written earlier in the same
    // call, so nothing has to start at zero.
    return bssn_rhs(in, out, shape, params, nullptr, scratch, sizeof(double) * kScratchValues, stream);
}
