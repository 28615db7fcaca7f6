// Wave diagnostics of Cartesian patches (JAX_BSSN/diagnostics/waves.py):
//   h_plus                         the plus-polarised physical metric
//                                  perturbation (waves.py:11-20), bit-identical
//                                  to the float64 reference;
//   composite wave norm sums       per level, over active vertices not covered by
//                                  a child of that level: sum of squares and max
//                                  |.| of h_plus minus the exact plane wave, sum
//                                  of H^2 and of |M|^2, and the vertex count
//                                  (waves.py:43-91).  Block partials in a fixed
//                                  order, folded by one block (deterministic).
#include <algorithm>
#include <cstring>
#include <string>

#include <cuda_runtime.h>

#include "../../include/bssn_gb300.h"
#include "bssn_driver.h"
#include "bssn_profile.h"

namespace bssn {
namespace {

constexpr int kWaveThreads = 256;
constexpr int kWaveBlocks = 304;  // two per SM on 152 SMs
constexpr int kWaveSums = 5;      // err^2, max |err|, H^2, |M|^2, count
constexpr int kMaxCovered = 8;

// 0.5 * (gt_yy / W^2 - gt_zz / W^2) with the reference's roundings.
__global__ void k_h_plus(const double* __restrict__ metric, const double* __restrict__ factor,
                         double* __restrict__ out, long long npts) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= npts) return;
    const double w2 = __dmul_rn(factor[t], factor[t]);
    const double yy = __ddiv_rn(metric[4 * npts + t], w2);
    const double zz = __ddiv_rn(metric[8 * npts + t], w2);
    out[t] = 0.5 * __dadd_rn(yy, -zz);
}

struct Covered {
    int count;
    int lo[kMaxCovered][3], hi[kMaxCovered][3];  // inclusive active indices
};

__device__ __forceinline__ bool is_covered(const Covered& C, int x, int y, int z) {
    for (int b = 0; b < C.count; ++b)
        if (x >= C.lo[b][0] && x <= C.hi[b][0] && y >= C.lo[b][1] && y <= C.hi[b][1] && z >= C.lo[b][2] &&
            z <= C.hi[b][2])
            return true;
    return false;
}

__global__ void __launch_bounds__(kWaveThreads)
k_wave_partial(const double* __restrict__ h, const double* __restrict__ coord, const double* __restrict__ H,
               const double* __restrict__ M, int n0, int n1, int n2, Covered C, double time, double amplitude,
               double wavelength, double* __restrict__ part) {
    const long long npts = (long long)n0 * n1 * n2;
    __shared__ double sh[kWaveSums][kWaveThreads];
    double acc[kWaveSums] = {0.0, 0.0, 0.0, 0.0, 0.0};
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < npts;
         t += (long long)gridDim.x * blockDim.x) {
        const int x = (int)(t / ((long long)n1 * n2));
        const long long r = t - (long long)x * n1 * n2;
        const int y = (int)(r / n2);
        const int z = (int)(r - (long long)y * n2);
        if (is_covered(C, x, y, z)) continue;
        // amplitude * sin(2 pi (x - t) / lambda), in the reference's order
        const double exact = amplitude * sin(2.0 * 3.141592653589793 * (coord[t] - time) / wavelength);
        const double err = h[t] - exact;
        acc[0] += err * err;
        acc[1] = fmax(acc[1], fabs(err));
        acc[2] += H[t] * H[t];
        acc[3] += M[t] * M[t] + M[npts + t] * M[npts + t] + M[2 * npts + t] * M[2 * npts + t];
        acc[4] += 1.0;
    }
#pragma unroll
    for (int q = 0; q < kWaveSums; ++q) sh[q][threadIdx.x] = acc[q];
    __syncthreads();
    for (int stride = kWaveThreads / 2; stride > 0; stride >>= 1) {
        if ((int)threadIdx.x < stride)
#pragma unroll
            for (int q = 0; q < kWaveSums; ++q) {
                const double o = sh[q][threadIdx.x + stride];
                sh[q][threadIdx.x] = (q == 1) ? fmax(sh[q][threadIdx.x], o) : sh[q][threadIdx.x] + o;
            }
        __syncthreads();
    }
    if (threadIdx.x == 0)
#pragma unroll
        for (int q = 0; q < kWaveSums; ++q) part[blockIdx.x * kWaveSums + q] = sh[q][0];
}

__global__ void k_wave_fold(const double* __restrict__ part, int nparts, double* __restrict__ out) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    double s[kWaveSums] = {0.0, 0.0, 0.0, 0.0, 0.0};
    for (int b = 0; b < nparts; ++b)
        for (int q = 0; q < kWaveSums; ++q)
            s[q] = (q == 1) ? fmax(s[q], part[b * kWaveSums + q]) : s[q] + part[b * kWaveSums + q];
    for (int q = 0; q < kWaveSums; ++q) out[q] = s[q];
}

}  // namespace
}  // namespace bssn

using namespace bssn;

extern "C" {

int bssn_h_plus(const BssnFields* state, const int32_t shape[3], double* h_plus, void* stream) {
    if (!state || !state->conformal_metric || !state->conformal_factor || !h_plus)
        return fail(BSSN_ERR_INVALID, "bssn_h_plus: null pointer");
    if (!shape || shape[0] < 1 || shape[1] < 1 || shape[2] < 1)
        return fail(BSSN_ERR_INVALID, "array extents must be positive");
    const long long npts = (long long)shape[0] * shape[1] * shape[2];
    BSSN_LAUNCH(KC_CONSTRAINTS, k_h_plus, (unsigned)((npts + 255) / 256), 256, (cudaStream_t)stream,
                state->conformal_metric, state->conformal_factor, h_plus, npts);
    return cuda_status(cudaGetLastError(), "bssn_h_plus");
}

size_t bssn_wave_norm_workspace_bytes(void) { return (size_t)kWaveBlocks * kWaveSums * sizeof(double); }

int bssn_wave_norm_sums(const double* h_plus, const double* coordinates, const double* hamiltonian,
                        const double* momentum, const int32_t shape[3], const int32_t* covered,
                        int32_t ncovered, double time, double amplitude, double wavelength, double* sums,
                        void* workspace, size_t workspace_bytes, void* stream) {
    if (!h_plus || !coordinates || !hamiltonian || !momentum || !sums)
        return fail(BSSN_ERR_INVALID, "bssn_wave_norm_sums: null pointer");
    if (!shape || shape[0] < 1 || shape[1] < 1 || shape[2] < 1)
        return fail(BSSN_ERR_INVALID, "array extents must be positive");
    if (ncovered < 0 || ncovered > kMaxCovered || (ncovered > 0 && !covered))
        return fail(BSSN_ERR_INVALID, "bssn_wave_norm_sums: between 0 and 8 covered boxes per level");
    if (!workspace || workspace_bytes < bssn_wave_norm_workspace_bytes())
        return fail(BSSN_ERR_WORKSPACE, "workspace missing or smaller than bssn_wave_norm_workspace_bytes()");
    Covered C;
    std::memset(&C, 0, sizeof(C));
    C.count = ncovered;
    for (int b = 0; b < ncovered; ++b)
        for (int a = 0; a < 3; ++a) {
            C.lo[b][a] = covered[6 * b + a];
            C.hi[b][a] = covered[6 * b + 3 + a];
        }
    cudaStream_t s = (cudaStream_t)stream;
    double* part = static_cast<double*>(workspace);
    BSSN_LAUNCH(KC_CONSTRAINTS, k_wave_partial, kWaveBlocks, kWaveThreads, s, h_plus, coordinates, hamiltonian,
                momentum, shape[0], shape[1], shape[2], C, time, amplitude, wavelength, part);
    BSSN_LAUNCH(KC_CONSTRAINTS, k_wave_fold, 1, 32, s, part, kWaveBlocks, sums);
    return cuda_status(cudaGetLastError(), "bssn_wave_norm_sums");
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Output staging (JAX_BSSN/diagnostics/openpmd.py:51-71, 254-285): the owned
// (ghost-stripped) box of every field copied, box after box, into one
// contiguous buffer, so that a writer needs a single device-to-host transfer.
// ---------------------------------------------------------------------------
namespace bssn {
namespace {

constexpr int kMaxGatherBoxes = BSSN_MAX_GATHER_BOXES;

struct GatherTable {
    int count;
    const double* src[kMaxGatherBoxes];
    int shape[kMaxGatherBoxes][3];
    int lo[kMaxGatherBoxes][3];
    int ext[kMaxGatherBoxes][3];
    long long offset[kMaxGatherBoxes];
};

__global__ void k_gather_boxes(GatherTable T, double* __restrict__ dst) {
    const int b = blockIdx.y;
    const long long n = (long long)T.ext[b][0] * T.ext[b][1] * T.ext[b][2];
    const double* src = T.src[b];
    double* out = dst + T.offset[b];
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
        const long long plane = (long long)T.ext[b][1] * T.ext[b][2];
        const int i = (int)(t / plane);
        const long long r = t - (long long)i * plane;
        const int j = (int)(r / T.ext[b][2]);
        const int k = (int)(r - (long long)j * T.ext[b][2]);
        out[t] = src[((long long)(T.lo[b][0] + i) * T.shape[b][1] + (T.lo[b][1] + j)) * T.shape[b][2] + T.lo[b][2] + k];
    }
}

}  // namespace
}  // namespace bssn

extern "C" int bssn_gather_boxes(int32_t count, const BssnBox* boxes, double* dst, void* stream) {
    using namespace bssn;
    if (count < 0 || count > kMaxGatherBoxes)
        return fail(BSSN_ERR_INVALID, "bssn_gather_boxes: between 0 and " + std::to_string(kMaxGatherBoxes) + " boxes");
    if (count == 0) return BSSN_OK;
    if (!boxes || !dst) return fail(BSSN_ERR_INVALID, "bssn_gather_boxes: null pointer");
    GatherTable T;
    std::memset(&T, 0, sizeof(T));
    T.count = count;
    long long offset = 0, largest = 0;
    for (int b = 0; b < count; ++b) {
        const BssnBox& x = boxes[b];
        if (!x.src) return fail(BSSN_ERR_INVALID, "bssn_gather_boxes: null source");
        long long n = 1;
        for (int a = 0; a < 3; ++a) {
            if (x.shape[a] < 1 || x.extent[a] < 0 || x.lo[a] < 0 || x.lo[a] + x.extent[a] > x.shape[a])
                return fail(BSSN_ERR_INVALID, "bssn_gather_boxes: box outside its array");
            T.shape[b][a] = x.shape[a];
            T.lo[b][a] = x.lo[a];
            T.ext[b][a] = x.extent[a];
            n *= x.extent[a];
        }
        T.src[b] = x.src;
        T.offset[b] = offset;
        offset += n;
        largest = n > largest ? n : largest;
    }
    if (largest == 0) return BSSN_OK;
    const unsigned bx = (unsigned)std::min<long long>((largest + 255) / 256, 1024);
    BSSN_LAUNCH(KC_EXPORT, k_gather_boxes, dim3(bx, count), 256, (cudaStream_t)stream, T, dst);
    return cuda_status(cudaGetLastError(), "bssn_gather_boxes");
}
