// Internal host-side interface between the C ABI and the kernel launchers.
#pragma once

#include <string>

#include <cuda_runtime.h>

#include "bssn_fields.cuh"

namespace bssn {

struct Box;

// Device scratch of one RHS evaluation on a patch (component stride Geo::cs).
struct RhsWork {
    double* d1 = nullptr;    // inner first derivatives: 3 * (NMIX [+ NMIX_MOM]) blocks
    double* der = nullptr;   // kappa != 0: gt^ij, B_i^j, B_i^j/W (24 blocks)
    double* damp = nullptr;  // kappa != 0: constraint-damping term for At (6 blocks)
    // FP32-arithmetic form, carved from the same memory (a launch uses one form):
    float* uf = nullptr;     // float perturbations of the state (21 blocks)
    float* d1f = nullptr;    // first derivatives
    float* derf = nullptr;   // derived fields (kappa != 0)
    float* dampf = nullptr;  // damping term (kappa != 0)
    // Matter sources (null: vacuum): kMatterComps padded blocks -- rho, S_i,
    // upper triangle of S_ij -- in the state's geometry.
    const double* mat = nullptr;
};

constexpr int kMatterComps = 10;

// Padded blocks of RHS scratch (RhsWork): the inner first derivatives of the
// NMIX base fields, plus, when kappa != 0, those of the NMIX_MOM momentum
// fields, 24 derived-field blocks and 6 damping blocks.
constexpr size_t rhs_work_blocks(bool with_mom) {
    return with_mom ? (size_t)(3 * (NMIX + NMIX_MOM) + 24 + 6) : (size_t)(3 * NMIX);
}
RhsWork carve_rhs_work(double* base, long long cs, bool with_mom);

cudaError_t launch_rhs(const double* u, double* k, const RhsWork& w, const Geo& G, const Box& box,
                       cudaStream_t stream);

// The reference's At and gt lower triangles minus their upper ones (6
// components: At xy, xz, yz, then gt xy, xz, yz), zero off the closure-row
// shell of the owned box: the step's values in FP64 (6 blocks), and in FP32
// the RK4 accumulator and two stage-value buffers (6 blocks each; stage[1]
// holds the FP32 copy of delta between steps).
struct LowerTriangle {
    double* delta = nullptr;
    float* acc = nullptr;
    float* stage[2] = {nullptr, nullptr};
};
constexpr size_t kLowerTriangleBlocks = 6 + 18 / 2;   // in FP64 blocks

// FP64 form with Sommerfeld faces: RK4 stage `stage` of the lower-triangle
// differences on the shell of `box` (first-order rates; reads w.d1 of the RHS
// just evaluated on u).  Reads lower_triangle_input(lt, q) at the stencil taps
// and writes lower_triangle_output(lt, q): the next stage's values, or after
// stage 4 (which also updates delta) delta's FP32 copy.
cudaError_t launch_lower_triangle(const double* u, const RhsWork& w, const LowerTriangle& lt, const Geo& G,
                                  const Box& box, int stage, cudaStream_t stream);
inline float* lower_triangle_input(const LowerTriangle& lt, int stage) {
    return lt.stage[(stage == 1 || stage == 3) ? 1 : 0];
}
inline float* lower_triangle_output(const LowerTriangle& lt, int stage) {
    return lt.stage[(stage == 1 || stage == 3) ? 0 : 1];
}

// The float forms' TMA kernels, by bit (kTmaGauge, kTmaDerivs, kTmaAt, kTmaKgt): each runs
// wherever its geometry allows when its bit is set (the derivatives by
// default), else the generic kernel; the number of tile waits that gave up
// since the last read, reset by reading; the TMA launches so far.
constexpr int kTmaGauge = 1, kTmaDerivs = 2, kTmaAt = 4, kTmaKgt = 8, kTmaAll = 15;
void set_tma_kernels(int mask);
cudaError_t tma_timeouts(int* count);
long long tma_launches();

// Launch-shape autotuning of the RHS of one geometry: times `reps` RHS
// evaluations per candidate block size of each launch slot and records the
// fastest for later launches of that slot at that size when its time is below
// `margin` x the current shapes' time (synchronises `stream`; refuses a
// capturing stream).  A summary is appended to *report when given.
cudaError_t tune_rhs(const double* u, double* k, const RhsWork& w, const Geo& G, const Box& box, cudaStream_t s,
                     int reps, float margin, std::string* report);

// First derivatives of the NMIX fields (3 * NMIX blocks of d1, layout
// d1[(d * NMIX + f) * cs + p]) on the box grown by the reach of the composed
// mixed derivatives (closed axes are not grown), for an FP64 geometry with
// kappa = 0: the inner factors the RHS kernels differentiate again.
cudaError_t launch_inner_derivs(const double* u, double* d1, const Geo& G, const Box& box, cudaStream_t stream);

// FP32 form with w.uf already holding the float perturbations of the whole
// padded block, about the backgrounds the FP32 RHS assumes (1 for the metric
// diagonal, W and alpha; one sample's value for the shift and K; 0 else).
// u supplies the FP64 values the FP32 kernels read: every component on the
// box, W wherever the momentum-constraint derived fields are formed.
cudaError_t launch_rhs_f32_prepared(const double* u, double* k, const RhsWork& w, const Geo& G, const Box& box,
                                    cudaStream_t stream);

// H, M_i (3 blocks), det-1, tr At, Gamma constraint (3 blocks) on the box,
// each block box.count long in the box's linear order.  Uses w.d1 (NMIX set)
// and w.der.
cudaError_t launch_constraints(const double* u, const RhsWork& w, const Geo& G, const Box& box, double* H,
                               double* M, double* detm1, double* trA, double* gam, cudaStream_t stream);

}  // namespace bssn
