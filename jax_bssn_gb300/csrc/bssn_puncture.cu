// Bowen-York puncture initial data (JAX_BSSN/utilities/bowen_york_solver.py):
//   puncture fields     Brill-Lindquist psi (:52-63), the conformal Bowen-York
//                       curvature (:66-91) and its flat contraction (:93-101)
//                       at given grid coordinates, in the reference's operation
//                       order;
//   pointwise/stencil   the seven-point and axisymmetric Laplacians (:104-148),
//   operators           the Hamiltonian source and its linearisation (:151-162),
//                       the linearised operators (:165-198) and the residuals
//                       (:201-230), each in the reference's operation order;
//   Newton solve        solve_conformal_factor (:283-366) with conjugate
//                       gradients on the Cartesian grid, and
//                       solve_axisymmetric_conformal_factor (:369-479) with
//                       BiCGSTAB on the meridional grid.
//
// The Krylov iterations of the reference come from jax.scipy.sparse.linalg
// (JAX >= 0.9.2, not part of the reference checkout): textbook conjugate
// gradients (Hestenes-Stiefel) and BiCGSTAB (van der Vorst 1992), started from
// zero, stopping once r.r <= max(tol^2 b.b, atol^2) or after maxiter
// iterations; BiCGSTAB also stops early when s.s < that bound and on
// breakdown (rho, alpha or omega zero).  Here every iteration is a few
// kernels on the caller's stream with no host round trip: each kernel's blocks
// write partial dot products, the last block to finish (a ticket counter, no
// waiting) folds them in a fixed order and updates a small control record that
// the next kernel reads; kernels launched after convergence return at once.
// The host reads the control record once per chunk of iterations and once per
// Newton step (the residual history).  Dot products are folded in a fixed
// order, so a solve is deterministic run to run.
//
// Storage: every vector spans the full grid (the reference's padded shape);
// unknowns live at the interior cells and the fixed outer cells hold zero, so
// stencils read zero-valued neighbours with no branches.  Inside the Krylov
// loop the Laplacian multiplies by 1/dx^2 instead of dividing; the operators
// exported on their own keep the reference's divisions.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/bssn_gb300.h"
#include "bssn_driver.h"
#include "bssn_profile.h"

#include <map>

namespace bssn {
namespace {

constexpr int kPunctThreads = 256;
constexpr int kMaxPunctures = BSSN_MAX_PUNCTURES;
constexpr int kMaxSums = 4;              // dot products folded per kernel
constexpr int kMaxApplyBlocks = 152 * 16; // cap of the persistent operator grid
constexpr int kUpdateBlocks = 152 * 4;   // grid of the vector-update kernels
constexpr int kChunk = 16;               // Krylov iterations enqueued between host checks (even)

static inline unsigned pblocks(long long n) { return (unsigned)((n + kPunctThreads - 1) / kPunctThreads); }

struct Punctures {
    int n;
    double m[kMaxPunctures];
    double x[kMaxPunctures][3];
    double p[kMaxPunctures][3];
};

// ---------------------------------------------------------------------------
// puncture fields (bowen_york_solver.py:52-101)
// ---------------------------------------------------------------------------
__global__ void k_puncture_fields(const double* __restrict__ grid, long long npts, Punctures P,
                                  double* __restrict__ psi_bl, double* __restrict__ curvature,
                                  double* __restrict__ curvature_squared) {
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < npts;
         t += (long long)gridDim.x * blockDim.x) {
        const double g[3] = {grid[3 * t], grid[3 * t + 1], grid[3 * t + 2]};
        double bl = 0.0;
        double K[9] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
        for (int a = 0; a < P.n; ++a) {
            double d[3];
#pragma unroll
            for (int i = 0; i < 3; ++i) d[i] = __dadd_rn(g[i], -P.x[a][i]);
            const double rsq = __dadd_rn(__dadd_rn(__dmul_rn(d[0], d[0]), __dmul_rn(d[1], d[1])), __dmul_rn(d[2], d[2]));
            const double r = __dsqrt_rn(rsq);
            const double term = __ddiv_rn(P.m[a], __dmul_rn(2.0, r));
            bl = a == 0 ? term : __dadd_rn(bl, term);
            double nrm[3];
#pragma unroll
            for (int i = 0; i < 3; ++i) nrm[i] = __ddiv_rn(d[i], r);
            const double pdn =
                __dadd_rn(__dadd_rn(__dmul_rn(P.p[a][0], nrm[0]), __dmul_rn(P.p[a][1], nrm[1])), __dmul_rn(P.p[a][2], nrm[2]));
            const double c = __ddiv_rn(3.0, __dmul_rn(2.0, __dmul_rn(r, r)));
#pragma unroll
            for (int i = 0; i < 3; ++i)
#pragma unroll
                for (int j = 0; j < 3; ++j) {
                    const double pn = __dadd_rn(__dmul_rn(P.p[a][i], nrm[j]), __dmul_rn(nrm[i], P.p[a][j]));
                    const double tr = __dadd_rn(i == j ? 1.0 : 0.0, -__dmul_rn(nrm[i], nrm[j]));
                    const double v = __dmul_rn(c, __dadd_rn(pn, -__dmul_rn(tr, pdn)));
                    K[3 * i + j] = a == 0 ? v : __dadd_rn(K[3 * i + j], v);
                }
        }
        if (psi_bl) psi_bl[t] = __dadd_rn(1.0, bl);
        if (curvature)
#pragma unroll
            for (int q = 0; q < 9; ++q) curvature[9 * t + q] = K[q];
        if (curvature_squared) {
            double s = __dmul_rn(K[0], K[0]);
#pragma unroll
            for (int q = 1; q < 9; ++q) s = __dadd_rn(s, __dmul_rn(K[q], K[q]));
            curvature_squared[t] = s;
        }
    }
}

__global__ void k_contract(const double* __restrict__ curvature, long long npts, double* __restrict__ out) {
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < npts;
         t += (long long)gridDim.x * blockDim.x) {
        double s = __dmul_rn(curvature[9 * t], curvature[9 * t]);
#pragma unroll
        for (int q = 1; q < 9; ++q) s = __dadd_rn(s, __dmul_rn(curvature[9 * t + q], curvature[9 * t + q]));
        out[t] = s;
    }
}

// psi^-7 and psi^-8 as integer powers: binary powering, then one reciprocal
__device__ __forceinline__ double inv_pow7(double x) {
    const double x2 = __dmul_rn(x, x), x3 = __dmul_rn(x2, x), x4 = __dmul_rn(x2, x2);
    return __ddiv_rn(1.0, __dmul_rn(x3, x4));
}
__device__ __forceinline__ double inv_pow8(double x) {
    const double x2 = __dmul_rn(x, x), x4 = __dmul_rn(x2, x2);
    return __ddiv_rn(1.0, __dmul_rn(x4, x4));
}

// S = 1/8 A^2 psi^-7 and dS = -7/8 A^2 psi^-8 (:151-162), left to right
__device__ __forceinline__ double source_of(double psi, double a2) {
    return __dmul_rn(__dmul_rn(0.125, a2), inv_pow7(psi));
}
__device__ __forceinline__ double lin_coefficient(double psi, double a2) {
    return __dmul_rn(__dmul_rn(-0.875, a2), inv_pow8(psi));
}

// ---------------------------------------------------------------------------
// Grids.  Cartesian: full extent n[0] x n[1] x n[2], unknowns at 1..n-2 on
// every axis.  Axisymmetric: n = (Nrho, 1, Nz), unknowns at rho 0..Nrho-2 and
// z 1..Nz-2; the regular ghost u(-dx/2) = u(dx/2) closes the axis.
// ---------------------------------------------------------------------------
struct SolveGrid {
    int n[3];
    int axi;
    double dx, dx2, inv_dx2;
    __host__ __device__ long long size() const { return (long long)n[0] * n[1] * n[2]; }
    __host__ __device__ bool interior(int i, int j, int k) const {
        if (axi) return i <= n[0] - 2 && k >= 1 && k <= n[2] - 2;
        return i >= 1 && i <= n[0] - 2 && j >= 1 && j <= n[1] - 2 && k >= 1 && k <= n[2] - 2;
    }
    __host__ __device__ long long unknowns() const {
        if (axi) return (long long)(n[0] - 1) * (n[2] - 2);
        return (long long)(n[0] - 2) * (n[1] - 2) * (n[2] - 2);
    }
};

__device__ __forceinline__ void decompose(const SolveGrid& G, long long t, int& i, int& j, int& k) {
    const long long plane = (long long)G.n[1] * G.n[2];
    i = (int)(t / plane);
    const long long r = t - (long long)i * plane;
    j = (int)(r / G.n[2]);
    k = (int)(r - (long long)j * G.n[2]);
}

// Reference-order Laplacians at an interior cell of a full-grid vector whose
// fixed cells are zero (exported operators and the Newton residual).
template <class F>
__device__ __forceinline__ double laplacian_exact(const SolveGrid& G, int i, int j, int k, F f) {
    if (G.axi) {
        const double c = f(i, 0, k);
        const double rp = f(i + 1, 0, k);
        const double rm = i == 0 ? c : f(i - 1, 0, k);
        const double rho = __dmul_rn(__dadd_rn((double)i, 0.5), G.dx);
        const double c2 = __dmul_rn(2.0, c);
        const double radial_second = __ddiv_rn(__dadd_rn(__dadd_rn(rp, -c2), rm), G.dx2);
        const double radial_first = __ddiv_rn(__dadd_rn(rp, -rm), __dmul_rn(__dmul_rn(2.0, rho), G.dx));
        const double axial_second = __ddiv_rn(__dadd_rn(__dadd_rn(f(i, 0, k + 1), f(i, 0, k - 1)), -c2), G.dx2);
        return __dadd_rn(__dadd_rn(radial_second, radial_first), axial_second);
    }
    double s = __dadd_rn(f(i + 1, j, k), f(i - 1, j, k));
    s = __dadd_rn(s, f(i, j + 1, k));
    s = __dadd_rn(s, f(i, j - 1, k));
    s = __dadd_rn(s, f(i, j, k + 1));
    s = __dadd_rn(s, f(i, j, k - 1));
    return __ddiv_rn(__dadd_rn(s, -__dmul_rn(6.0, f(i, j, k))), G.dx2);
}

// ---------------------------------------------------------------------------
// Exported operators (:104-230) on the reference's shapes.  Inputs/outputs of
// the Laplacian and linearised operators are interior-shaped; they are
// evaluated on a zero-padded full-grid copy.
// ---------------------------------------------------------------------------
__global__ void k_pad_interior(const double* __restrict__ in, SolveGrid G, double* __restrict__ full) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= G.size()) return;
    int i, j, k;
    decompose(G, t, i, j, k);
    double v = 0.0;
    if (G.interior(i, j, k)) {
        if (G.axi) v = in[(long long)i * (G.n[2] - 2) + (k - 1)];
        else v = in[((long long)(i - 1) * (G.n[1] - 2) + (j - 1)) * (G.n[2] - 2) + (k - 1)];
    }
    full[t] = v;
}

// op 0: Laplacian; op 1: linearised operator Lap(d) + dS(psi, A2) d;
// op 2: residual Lap(u) + S(psi_bl + u, A2) with full-grid psi_bl and A2.
// For ops 0/1, psi and A2 are interior-shaped.
__global__ void k_operator(const double* __restrict__ full, const double* __restrict__ b, const double* __restrict__ c,
                           SolveGrid G, int op, double* __restrict__ out) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= G.size()) return;
    int i, j, k;
    decompose(G, t, i, j, k);
    if (!G.interior(i, j, k)) return;
    const long long plane = (long long)G.n[1] * G.n[2];
    auto f = [&](int x, int y, int z) { return full[(long long)x * plane + (long long)y * G.n[2] + z]; };
    const long long o = G.axi ? (long long)i * (G.n[2] - 2) + (k - 1)
                              : ((long long)(i - 1) * (G.n[1] - 2) + (j - 1)) * (G.n[2] - 2) + (k - 1);
    const double lap = laplacian_exact(G, i, j, k, f);
    double v = lap;
    if (op == 1) v = __dadd_rn(lap, __dmul_rn(lin_coefficient(b[o], c[o]), f(i, j, k)));
    if (op == 2) v = __dadd_rn(lap, source_of(__dadd_rn(b[t], f(i, j, k)), c[t]));
    out[o] = v;
}

__global__ void k_pointwise(const double* __restrict__ a, const double* __restrict__ b, const double* __restrict__ c,
                            long long n, int op, double* __restrict__ out) {
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x)
        out[t] = op == 0 ? source_of(a[t], b[t]) : __dmul_rn(lin_coefficient(b[t], c[t]), a[t]);
}

// ---------------------------------------------------------------------------
// Solver control record and deterministic block folds
// ---------------------------------------------------------------------------
struct SolveCtrl {
    double gamma;        // r.r of the current iterate
    double alpha, beta, omega, rho;
    double atol2;        // stopping bound on r.r
    double bb;           // b.b of the Newton residual
    double rms;          // Newton residual RMS
    int k, maxiter, done, first;
    int bad_psi, bad_u;  // Newton-level checks (axisymmetric solve)
    unsigned ticket;
    int pad;
};

// Block sum of NS values in a fixed order (warp shuffles, then warp 0).
template <int NS>
__device__ __forceinline__ void block_sums(double (&v)[NS], double (*shared)[32]) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int nwarps = (blockDim.x + 31) >> 5;
#pragma unroll
    for (int q = 0; q < NS; ++q) {
        double s = v[q];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
        if (lane == 0) shared[q][warp] = s;
    }
    __syncthreads();
    if (warp == 0) {
#pragma unroll
        for (int q = 0; q < NS; ++q) {
            double s = lane < nwarps ? shared[q][lane] : 0.0;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
            v[q] = s;
        }
    }
}

// Writes this block's partials; returns true in the one block that finishes
// last, in which every thread then holds the fixed-order fold of all blocks'
// partials in `tot` (thread 0's copy is the one used).
template <int NS>
__device__ bool fold_last(double (&v)[NS], double* __restrict__ partial, unsigned* ticket, double (&tot)[NS]) {
    __shared__ double sh[NS][32];
    __shared__ bool last;
    const unsigned nblocks = gridDim.x * gridDim.y * gridDim.z;
    const unsigned bid = blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z);
    const int tid = threadIdx.x;
    block_sums<NS>(v, sh);
    if (tid == 0) {
#pragma unroll
        for (int q = 0; q < NS; ++q) partial[(long long)bid * NS + q] = v[q];
        __threadfence();
        last = atomicAdd(ticket, 1u) == nblocks - 1;
    }
    __syncthreads();
    if (!last) return false;
    __threadfence();
    double s[NS];
#pragma unroll
    for (int q = 0; q < NS; ++q) s[q] = 0.0;
    for (unsigned b = tid; b < nblocks; b += blockDim.x)
#pragma unroll
        for (int q = 0; q < NS; ++q) s[q] += __ldcg(partial + (long long)b * NS + q);
    __syncthreads();
    block_sums<NS>(s, sh);
#pragma unroll
    for (int q = 0; q < NS; ++q) tot[q] = s[q];
    if (tid == 0) *ticket = 0u;
    return true;
}

__device__ __forceinline__ SolveCtrl read_ctrl(const SolveCtrl* c) {
    SolveCtrl r;
    const double* d = reinterpret_cast<const double*>(c);
#pragma unroll
    for (int q = 0; q < (int)(sizeof(SolveCtrl) / sizeof(double)); ++q)
        reinterpret_cast<double*>(&r)[q] = __ldcg(d + q);
    return r;
}

// ---------------------------------------------------------------------------
// Newton level: residual F(u) = Lap(u) + S(psi_bl + u) at the interior (zero at
// fixed cells), its RMS, and the Krylov start.  The Krylov solve runs on the
// system scaled by dx^2 (the same solution; every stopping test is scale
// free): b = dx^2 F, and the operator's centre coefficient dx^2 dS/du - 6
// (Cartesian) or dx^2 dS/du - 4 (meridional) is stored per cell, so that one
// operator application is a neighbour sum and one FMA.  x = 0 comes from a
// memset; r = rhat = b.  Conjugate gradients run on the negated system
// (-A) x = -b: every iterate is the exact negation of the standard one (x
// itself is unchanged, bit for bit), and the operator needs no negation.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kPunctThreads)
k_newton_residual(const double* __restrict__ u, const double* __restrict__ psi_bl, const double* __restrict__ a2,
                  SolveGrid G, double* __restrict__ r, double* __restrict__ rhat, double* __restrict__ centre,
                  double* __restrict__ partial, SolveCtrl* ctrl, double tol2, int maxiter, int negate) {
    double acc[4] = {0.0, 0.0, 0.0, 0.0};   // F.F, nonpositive psi, nonfinite u, b.b
    const long long plane = (long long)G.n[1] * G.n[2];
    const double diag = G.axi ? 4.0 : 6.0;
    auto f = [&](int x, int y, int z) { return u[(long long)x * plane + (long long)y * G.n[2] + z]; };
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < G.size();
         t += (long long)gridDim.x * blockDim.x) {
        int i, j, k;
        decompose(G, t, i, j, k);
        double res = 0.0, b = 0.0, c = 0.0;
        if (G.interior(i, j, k)) {
            const double psi = __dadd_rn(psi_bl[t], u[t]);
            res = __dadd_rn(laplacian_exact(G, i, j, k, f), source_of(psi, a2[t]));
            b = G.dx2 * res;
            if (negate) b = -b;
            c = fma(G.dx2, lin_coefficient(psi, a2[t]), -diag);
            acc[0] += res * res;
            if (!(psi > 0.0)) acc[1] += 1.0;
            if (!isfinite(u[t])) acc[2] += 1.0;
            acc[3] += b * b;
        }
        r[t] = b;
        if (rhat) rhat[t] = b;
        centre[t] = c;
    }
    double tot[4];
    if (!fold_last<4>(acc, partial, &ctrl->ticket, tot)) return;
    if (threadIdx.x == 0) {
        const double bb = tot[3];
        ctrl->bb = bb;
        ctrl->gamma = bb;
        ctrl->rms = sqrt(tot[0] / (double)G.unknowns());
        ctrl->atol2 = tol2 * bb;
        ctrl->k = 0;
        ctrl->maxiter = maxiter;
        ctrl->first = 1;
        ctrl->alpha = ctrl->omega = 1.0;
        ctrl->rho = bb;   // rhat.r with rhat = r = b
        ctrl->beta = 0.0;
        ctrl->done = !(bb > ctrl->atol2 && maxiter > 0);
        ctrl->bad_psi = tot[1] > 0.0;
        ctrl->bad_u = tot[2] > 0.0;
    }
}

__global__ void k_newton_update(double* __restrict__ u, const double* __restrict__ x, long long n) {
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x)
        u[t] = u[t] + x[t];
}

__global__ void k_psi_total(const double* __restrict__ psi_bl, const double* __restrict__ u, double* __restrict__ psi,
                            long long n) {
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x)
        psi[t] = psi_bl[t] + u[t];
}

// ---------------------------------------------------------------------------
// Conjugate gradients on A = -dx^2 (Lap + dS) (Cartesian).  One iteration:
//   k_cg_apply   p = r + beta p_prev (p = r at the first), Bp, p.Bp with
//                B = -A = dx^2 (Lap + dS)  -> alpha = gamma / p.Bp
//   k_cg_update  r -= alpha Bp, r.r -> beta, gamma, k, done
// x += alpha p of an iteration is applied by the next iteration's operator
// kernel, which reads that p anyway (the same FMA on the same values, so x is
// unchanged bit for bit), and after the last iteration by k_cg_finish; the
// update kernel then streams 24 bytes per unknown instead of 48.
// The apply kernel stages p of one x plane of a 32 x 8 (z, y) tile in shared
// memory, with its one-cell halo, and marches along x carrying the x
// neighbours in registers, so each p value is formed once per tile (plus the
// halo) rather than once per stencil tap.  Its grid is persistent (the
// resident blocks of every SM): the (tile, plane) steps are split evenly
// between blocks, a block's range possibly continuing into the next tile, so
// that every SM gets the same FP64 work.  p ping-pongs between two buffers,
// since neighbouring tiles still read the previous p.
// ---------------------------------------------------------------------------
constexpr int kTz = 32, kTy = 8;

__global__ void __launch_bounds__(kTz* kTy)
k_cg_apply(const double* __restrict__ r, const double* __restrict__ pin, double* __restrict__ pout,
           const double* __restrict__ centre, double* __restrict__ ap, double* __restrict__ sol, SolveGrid G,
           SolveCtrl* ctrl, double* __restrict__ partial) {
    // two plane buffers: plane x+1 is written while plane x may still be read,
    // so each plane step needs one barrier
    __shared__ double tile[2][kTy + 2][kTz + 2];
    const SolveCtrl C = read_ctrl(ctrl);
    if (C.done) return;
    const bool first = C.first != 0;
    const double beta = C.beta;
    const int tz = threadIdx.x % kTz, ty = threadIdx.x / kTz;
    const int tiles_z = (G.n[2] - 2 + kTz - 1) / kTz;
    const int tiles_y = (G.n[1] - 2 + kTy - 1) / kTy;
    const int planes = G.n[0] - 2;
    const long long steps = (long long)tiles_z * tiles_y * planes;
    const long long w0 = steps * blockIdx.x / gridDim.x, w1 = steps * (blockIdx.x + 1) / gridDim.x;
    const long long sx = (long long)G.n[1] * G.n[2], sy = G.n[2];
    auto pnew = [&](long long idx) { return first ? r[idx] : fma(beta, pin[idx], r[idx]); };
    // halo roles: a row of the tile's y halo and/or a column of its z halo
    const int hy_row = ty == 0 ? 0 : ty == kTy - 1 ? kTy + 1 : -1;
    const int hz_col = tz == 0 ? 0 : tz == kTz - 1 ? kTz + 1 : -1;
    double dot[1] = {0.0};
    for (long long w = w0; w < w1;) {
        const int t = (int)(w / planes);
        const int xs = 1 + (int)(w - (long long)t * planes);
        const int xe = 1 + (int)min((long long)planes, (long long)(xs - 1) + (w1 - w));   // exclusive
        w += xe - xs;
        const int z = 1 + (t % tiles_z) * kTz + tz;
        const int y = 1 + (t / tiles_z) * kTy + ty;
        const bool in_yz = y <= G.n[1] - 1 && z <= G.n[2] - 1;   // y, z >= 1 by construction
        const bool interior = y <= G.n[1] - 2 && z <= G.n[2] - 2;
        const long long own = (long long)y * sy + z;
        // in-array halo cells of this thread (offset from `own`), or none
        const long long hy_off = hy_row == 0 ? -sy : sy;
        const bool hy_ok = hy_row >= 0 && z <= G.n[2] - 1 && (hy_row == 0 || y + 1 <= G.n[1] - 1);
        const long long hz_off = hz_col == 0 ? -1 : 1;
        const bool hz_ok = hz_col >= 0 && y <= G.n[1] - 1 && (hz_col == 0 || z + 1 <= G.n[2] - 1);
        auto own_at = [&](int x) { return in_yz ? pnew((long long)x * sx + own) : 0.0; };
        auto hy_at = [&](int x) { return hy_ok ? pnew((long long)x * sx + own + hy_off) : 0.0; };
        auto hz_at = [&](int x) { return hz_ok ? pnew((long long)x * sx + own + hz_off) : 0.0; };
        auto centre_at = [&](int x) { return interior ? centre[(long long)x * sx + own] : 0.0; };
        double pm = own_at(xs - 1), pc = own_at(xs), pn = own_at(xs + 1);
        double hy = hy_at(xs), hz = hz_at(xs), cc = centre_at(xs);
        int buf = 0;
        for (int x = xs; x < xe; ++x) {
            tile[buf][ty + 1][tz + 1] = pc;
            if (hy_row >= 0) tile[buf][hy_row][tz + 1] = hy;
            if (hz_col >= 0) tile[buf][ty + 1][hz_col] = hz;
            // loads of the next plane step, in flight across the barrier and the stencil
            double pnn = 0.0, hyn = 0.0, hzn = 0.0, ccn = 0.0;
            if (x + 1 < xe) {
                pnn = x + 2 <= G.n[0] - 1 ? own_at(x + 2) : 0.0;
                hyn = hy_at(x + 1);
                hzn = hz_at(x + 1);
                ccn = centre_at(x + 1);
            }
            __syncthreads();
            if (interior) {
                const long long o = (long long)x * sx + own;
                double s = pn + pm;
                s += tile[buf][ty + 2][tz + 1];
                s += tile[buf][ty][tz + 1];
                s += tile[buf][ty + 1][tz + 2];
                s += tile[buf][ty + 1][tz];
                const double a = fma(cc, pc, s);
                if (!first) sol[o] = fma(C.alpha, pin[o], sol[o]);   // x += alpha p of the previous iteration
                pout[o] = pc;
                ap[o] = a;
                dot[0] = fma(pc, a, dot[0]);
            }
            pm = pc;
            pc = pn;
            pn = pnn;
            hy = hyn;
            hz = hzn;
            cc = ccn;
            buf ^= 1;
        }
        __syncthreads();   // the next segment starts over in buffer 0
    }
    double tot[1];
    if (!fold_last<1>(dot, partial, &ctrl->ticket, tot)) return;
    if (threadIdx.x == 0) ctrl->alpha = C.gamma / tot[0];
}

// Two samples per thread and step (16-byte loads), two steps in flight.
__global__ void __launch_bounds__(kPunctThreads)
k_cg_update(double* __restrict__ r, const double* __restrict__ ap, long long n, SolveCtrl* ctrl,
            double* __restrict__ partial) {
    const SolveCtrl C = read_ctrl(ctrl);
    if (C.done) return;
    const double alpha = C.alpha;
    double rr[1] = {0.0};
    double rr1 = 0.0;
    const long long pairs = n / 2;
    const long long stride = (long long)gridDim.x * blockDim.x;
    double2* r2 = reinterpret_cast<double2*>(r);
    const double2* a2 = reinterpret_cast<const double2*>(ap);
#pragma unroll 2
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < pairs; t += stride) {
        const double2 av = a2[t], rv = r2[t];
        const double rx = fma(-alpha, av.x, rv.x), ry = fma(-alpha, av.y, rv.y);
        r2[t] = make_double2(rx, ry);
        rr[0] = fma(rx, rx, rr[0]);
        rr1 = fma(ry, ry, rr1);
    }
    if ((n & 1) && blockIdx.x == 0 && threadIdx.x == 0) {
        const long long t = n - 1;
        const double rn = fma(-alpha, ap[t], r[t]);
        r[t] = rn;
        rr1 = fma(rn, rn, rr1);
    }
    rr[0] += rr1;
    double tot[1];
    if (!fold_last<1>(rr, partial, &ctrl->ticket, tot)) return;
    if (threadIdx.x == 0) {
        ctrl->beta = tot[0] / C.gamma;
        ctrl->gamma = tot[0];
        ctrl->k = C.k + 1;
        ctrl->first = 0;
        ctrl->done = !(tot[0] > C.atol2 && C.k + 1 < C.maxiter);
    }
}

// x += alpha p of the last conjugate-gradient iteration
__global__ void k_cg_finish(double* __restrict__ x, const double* __restrict__ p, long long n,
                            const SolveCtrl* ctrl) {
    const double alpha = __ldcg(&ctrl->alpha);
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x)
        x[t] = fma(alpha, p[t], x[t]);
}

// ---------------------------------------------------------------------------
// BiCGSTAB on A = -dx^2 (Lap_axi + dS) (meridional grid).  With h_i = 1/(2i+1)
// = dx / (2 rho_i), A v = -((1 + h_i) v[i+1] + (1 - h_i) v[i-1] + v[k+1] +
// v[k-1] + c v), c the stored centre coefficient; 1 - h_0 = 0 closes the axis.
// One iteration:
//   k_bicg_p   p = r + beta (p_prev - omega q_prev) (p = r at the first),
//              q = A p, rhat.q -> alpha = rho / rhat.q
//   k_bicg_s   s = r - alpha q, t = A s, s.s, t.s, t.t -> omega, early exit
//   k_bicg_x   x += alpha p (+ omega s), r = s (- omega t), r.r, rhat.r
//              -> beta, rho, k, done (convergence, maxiter or breakdown)
// The two operator kernels stage the combined vector of a 32 x 8 (z, rho)
// tile plus halo in shared memory, one tile per block.
// ---------------------------------------------------------------------------
constexpr int kAz = 32, kAr = 8;

__device__ __forceinline__ double axi_apply_tile(double (*tile)[kAz + 2], const double* rows, int i, int ti, int tk,
                                                 double centre) {
    const double c = tile[ti + 1][tk + 1];
    const double rp = tile[ti + 2][tk + 1];
    const double rm = i == 0 ? c : tile[ti][tk + 1];
    const double zs = tile[ti + 1][tk + 2] + tile[ti + 1][tk];
    return -fma(rows[2 * ti], rp, fma(rows[2 * ti + 1], rm, fma(centre, c, zs)));
}

// 1 + h_i and 1 - h_i of the block's rows
__device__ __forceinline__ void axi_rows(double* rows, int i0) {
    if (threadIdx.x < kAr) {
        const double h = 1.0 / (double)(2 * (i0 + (int)threadIdx.x) + 1);
        rows[2 * threadIdx.x] = 1.0 + h;
        rows[2 * threadIdx.x + 1] = 1.0 - h;
    }
}

// Fills the (kAr + 2) x (kAz + 2) tile of vec(i, k) around the block's cells;
// cells outside the array read as zero.
template <class V>
__device__ __forceinline__ void axi_fill_tile(const SolveGrid& G, double (*tile)[kAz + 2], int i0, int k0, V vec) {
    for (int q = threadIdx.x; q < (kAr + 2) * (kAz + 2); q += blockDim.x) {
        const int ti = q / (kAz + 2), tk = q - ti * (kAz + 2);
        const int i = i0 - 1 + ti, k = k0 - 1 + tk;
        tile[ti][tk] = (i >= 0 && i <= G.n[0] - 1 && k >= 0 && k <= G.n[2] - 1) ? vec((long long)i * G.n[2] + k) : 0.0;
    }
}

__global__ void __launch_bounds__(kAz* kAr)
k_bicg_p(const double* __restrict__ r, const double* __restrict__ rhat, const double* __restrict__ pin,
         const double* __restrict__ qin, double* __restrict__ pout, double* __restrict__ qout,
         const double* __restrict__ centre, SolveGrid G, SolveCtrl* ctrl, double* __restrict__ partial) {
    __shared__ double tile[kAr + 2][kAz + 2];
    __shared__ double rows[2 * kAr];
    const SolveCtrl C = read_ctrl(ctrl);
    if (C.done) return;
    const bool first = C.first != 0;
    const double beta = C.beta, omega = C.omega;
    const int tk = threadIdx.x % kAz, ti = threadIdx.x / kAz;
    const int i0 = blockIdx.y * kAr, k0 = 1 + blockIdx.x * kAz;
    axi_rows(rows, i0);
    axi_fill_tile(G, tile, i0, k0, [&](long long o) { return first ? r[o] : fma(beta, fma(-omega, qin[o], pin[o]), r[o]); });
    __syncthreads();
    const int i = i0 + ti, k = k0 + tk;
    double acc[1] = {0.0};
    if (G.interior(i, 0, k)) {
        const long long o = (long long)i * G.n[2] + k;
        const double q = axi_apply_tile(tile, rows, i, ti, tk, centre[o]);
        pout[o] = tile[ti + 1][tk + 1];
        qout[o] = q;
        acc[0] = rhat[o] * q;
    }
    double tot[1];
    if (!fold_last<1>(acc, partial, &ctrl->ticket, tot)) return;
    if (threadIdx.x == 0) ctrl->alpha = C.rho / tot[0];
}

__global__ void __launch_bounds__(kAz* kAr)
k_bicg_s(const double* __restrict__ r, const double* __restrict__ q, double* __restrict__ s, double* __restrict__ tv,
         const double* __restrict__ centre, SolveGrid G, SolveCtrl* ctrl, double* __restrict__ partial) {
    __shared__ double tile[kAr + 2][kAz + 2];
    __shared__ double rows[2 * kAr];
    const SolveCtrl C = read_ctrl(ctrl);
    if (C.done) return;
    const double alpha = C.alpha;
    const int tk = threadIdx.x % kAz, ti = threadIdx.x / kAz;
    const int i0 = blockIdx.y * kAr, k0 = 1 + blockIdx.x * kAz;
    axi_rows(rows, i0);
    axi_fill_tile(G, tile, i0, k0, [&](long long o) { return fma(-alpha, q[o], r[o]); });
    __syncthreads();
    const int i = i0 + ti, k = k0 + tk;
    double acc[3] = {0.0, 0.0, 0.0};   // s.s, t.s, t.t
    if (G.interior(i, 0, k)) {
        const long long o = (long long)i * G.n[2] + k;
        const double sc = tile[ti + 1][tk + 1];
        const double tt = axi_apply_tile(tile, rows, i, ti, tk, centre[o]);
        s[o] = sc;
        tv[o] = tt;
        acc[0] = sc * sc;
        acc[1] = tt * sc;
        acc[2] = tt * tt;
    }
    double tot[3];
    if (!fold_last<3>(acc, partial, &ctrl->ticket, tot)) return;
    if (threadIdx.x == 0) {
        const bool early = tot[0] < C.atol2;
        ctrl->omega = early ? 0.0 : tot[1] / tot[2];
        ctrl->first = early ? -1 : 0;   // -1 marks the early exit for k_bicg_x
    }
}

__global__ void __launch_bounds__(kPunctThreads)
k_bicg_x(double* __restrict__ x, double* __restrict__ r, const double* __restrict__ rhat, const double* __restrict__ p,
         const double* __restrict__ s, const double* __restrict__ tv, long long n, SolveCtrl* ctrl,
         double* __restrict__ partial) {
    const SolveCtrl C = read_ctrl(ctrl);
    if (C.done) return;
    const bool early = C.first == -1;
    const double alpha = C.alpha, omega = C.omega;
    double acc[2] = {0.0, 0.0};   // r.r, rhat.r
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
        const double xa = fma(alpha, p[t], x[t]);
        double rn;
        if (early) {
            x[t] = xa;
            rn = s[t];
        } else {
            x[t] = fma(omega, s[t], xa);
            rn = fma(-omega, tv[t], s[t]);
        }
        r[t] = rn;
        acc[0] = fma(rn, rn, acc[0]);
        acc[1] = fma(rhat[t], rn, acc[1]);
    }
    double tot[2];
    if (!fold_last<2>(acc, partial, &ctrl->ticket, tot)) return;
    if (threadIdx.x == 0) {
        const int k = C.k + 1;
        const double rho = tot[1];
        const bool breakdown = (!early && (omega == 0.0 || alpha == 0.0)) || rho == 0.0;
        ctrl->beta = (rho / C.rho) * (alpha / omega);
        ctrl->rho = rho;
        ctrl->gamma = tot[0];
        ctrl->k = k;
        ctrl->first = 0;
        ctrl->done = early || breakdown || !(tot[0] > C.atol2 && k < C.maxiter);
    }
}

// ---------------------------------------------------------------------------
// workspace: 10 full-grid vectors, the partial sums, the control record
// ---------------------------------------------------------------------------
enum { V_R, V_RHAT, V_CENTRE, V_X, V_P0, V_P1, V_Q, V_S, V_T, V_Q1, V_COUNT };

int grid_of(const int32_t shape[3], int axi, double dx, SolveGrid& G) {
    if (!shape) return fail(BSSN_ERR_INVALID, "null shape");
    for (int a = 0; a < 3; ++a) G.n[a] = shape[a];
    G.axi = axi ? 1 : 0;
    if (G.axi) {
        if (shape[1] != 1 || shape[0] < 2 || shape[2] < 3)
            return fail(BSSN_ERR_INVALID, "grid requires at least two rho and three z cells");
    } else if (shape[0] < 3 || shape[1] < 3 || shape[2] < 3) {
        return fail(BSSN_ERR_INVALID, "every grid axis needs at least three cells");
    }
    if (!(dx > 0.0) || !std::isfinite(dx)) return fail(BSSN_ERR_INVALID, "dx must be finite and positive");
    G.dx = dx;
    G.dx2 = dx * dx;
    G.inv_dx2 = 1.0 / G.dx2;
    return BSSN_OK;
}

long long max_blocks(const SolveGrid& G) {
    long long apply = kMaxApplyBlocks;
    if (G.axi) apply = (long long)((G.n[2] - 2 + kAz - 1) / kAz) * ((G.n[0] - 1 + kAr - 1) / kAr);
    return std::max<long long>(apply, kUpdateBlocks);
}

size_t workspace_bytes(const SolveGrid& G) {
    const size_t vec = (size_t)G.size() * sizeof(double);
    const size_t vec_al = (vec + 255) & ~(size_t)255;
    return V_COUNT * vec_al + (size_t)max_blocks(G) * kMaxSums * sizeof(double) + 256 + sizeof(SolveCtrl);
}

unsigned update_blocks(long long n) { return (unsigned)std::min<long long>(pblocks(n), kUpdateBlocks); }

// A non-blocking stream per device and thread for the solve, ordered after
// and before the caller's stream with events (stream capture of the Krylov
// chunks needs a stream other than the legacy default stream).
struct SolveStream {
    cudaStream_t s = nullptr;
    cudaEvent_t in = nullptr, out = nullptr;
};

cudaError_t solve_stream(SolveStream*& out) {
    thread_local std::map<int, SolveStream> streams;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    SolveStream& ss = streams[dev];
    if (!ss.s) {
        e = cudaStreamCreateWithFlags(&ss.s, cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ss.in, cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ss.out, cudaEventDisableTiming);
        if (e != cudaSuccess) return e;
    }
    out = &ss;
    return cudaSuccess;
}

// Persistent grid of the Cartesian operator kernel: its resident blocks on
// every SM, at most one block per (tile, plane) step.
unsigned cg_apply_blocks(const SolveGrid& G) {
    int dev = 0, sms = 152, per_sm = 4;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_cg_apply, kTz * kTy, 0);
    const long long steps = (long long)((G.n[2] - 2 + kTz - 1) / kTz) * ((G.n[1] - 2 + kTy - 1) / kTy) * (G.n[0] - 2);
    const long long want = (long long)sms * std::max(per_sm, 1);
    return (unsigned)std::min<long long>(std::min<long long>(want, steps), kMaxApplyBlocks);
}

}  // namespace
}  // namespace bssn

using namespace bssn;

extern "C" {

int bssn_puncture_fields(const double* grid, int64_t npoints, const double* masses, const double* positions,
                         const double* momenta, int32_t npunctures, double* psi_bl, double* curvature,
                         double* curvature_squared, void* stream) {
    if (!grid || !masses || !positions || !momenta) return fail(BSSN_ERR_INVALID, "bssn_puncture_fields: null pointer");
    if (npunctures < 1 || npunctures > kMaxPunctures)
        return fail(BSSN_ERR_INVALID, "between 1 and " + std::to_string(kMaxPunctures) + " punctures");
    if (npoints < 0) return fail(BSSN_ERR_INVALID, "npoints must be non-negative");
    Punctures P;
    std::memset(&P, 0, sizeof(P));
    P.n = npunctures;
    for (int a = 0; a < npunctures; ++a) {
        P.m[a] = masses[a];
        for (int i = 0; i < 3; ++i) {
            P.x[a][i] = positions[3 * a + i];
            P.p[a][i] = momenta[3 * a + i];
        }
    }
    if (npoints == 0) return BSSN_OK;
    const unsigned blocks = (unsigned)std::min<long long>(pblocks(npoints), 152 * 16);
    BSSN_LAUNCH(KC_SOLVE_NEWTON, k_puncture_fields, blocks, kPunctThreads, (cudaStream_t)stream, grid, npoints, P,
                psi_bl, curvature, curvature_squared);
    return cuda_status(cudaGetLastError(), "bssn_puncture_fields");
}

int bssn_puncture_operator(int32_t op, const double* a, const double* b, const double* c, const int32_t shape[3],
                           double dx, int32_t axisymmetric, double* out, void* workspace, size_t workspace_bytes_,
                           void* stream) {
    cudaStream_t s = (cudaStream_t)stream;
    if (!a || !out) return fail(BSSN_ERR_INVALID, "bssn_puncture_operator: null pointer");
    if (op == BSSN_PUNCTURE_CONTRACT || op == BSSN_PUNCTURE_SOURCE || op == BSSN_PUNCTURE_LINEARIZED_SOURCE) {
        if (!shape || shape[0] < 0 || shape[1] < 0 || shape[2] < 0)
            return fail(BSSN_ERR_INVALID, "array extents must be non-negative");
        const long long n = (long long)shape[0] * shape[1] * shape[2];
        if (n == 0) return BSSN_OK;
        const unsigned blocks = (unsigned)std::min<long long>(pblocks(n), 152 * 16);
        if (op == BSSN_PUNCTURE_CONTRACT) {
            BSSN_LAUNCH(KC_SOLVE_NEWTON, k_contract, blocks, kPunctThreads, s, a, n, out);
        } else {
            if (!b || (op == BSSN_PUNCTURE_LINEARIZED_SOURCE && !c))
                return fail(BSSN_ERR_INVALID, "bssn_puncture_operator: null pointer");
            BSSN_LAUNCH(KC_SOLVE_NEWTON, k_pointwise, blocks, kPunctThreads, s, a, b, c, n,
                        op == BSSN_PUNCTURE_SOURCE ? 0 : 1, out);
        }
        return cuda_status(cudaGetLastError(), "bssn_puncture_operator");
    }
    if (op != BSSN_PUNCTURE_LAPLACIAN && op != BSSN_PUNCTURE_LINEARIZED_OPERATOR && op != BSSN_PUNCTURE_RESIDUAL)
        return fail(BSSN_ERR_INVALID, "unknown puncture operator");
    SolveGrid G;
    if (int e = grid_of(shape, axisymmetric, dx, G)) return e;
    if (op != BSSN_PUNCTURE_LAPLACIAN && (!b || !c)) return fail(BSSN_ERR_INVALID, "bssn_puncture_operator: null pointer");
    const long long n = G.size();
    const double* full = a;
    if (op != BSSN_PUNCTURE_RESIDUAL) {
        if (!workspace || workspace_bytes_ < (size_t)n * sizeof(double))
            return fail(BSSN_ERR_WORKSPACE, "workspace must hold one full-grid array");
        double* pad = static_cast<double*>(workspace);
        BSSN_LAUNCH(KC_SOLVE_NEWTON, k_pad_interior, pblocks(n), kPunctThreads, s, a, G, pad);
        full = pad;
    }
    const int code = op == BSSN_PUNCTURE_LAPLACIAN ? 0 : op == BSSN_PUNCTURE_LINEARIZED_OPERATOR ? 1 : 2;
    BSSN_LAUNCH(KC_SOLVE_NEWTON, k_operator, pblocks(n), kPunctThreads, s, full, b, c, G, code, out);
    return cuda_status(cudaGetLastError(), "bssn_puncture_operator");
}

size_t bssn_puncture_workspace_bytes(const int32_t shape[3], int32_t axisymmetric) {
    SolveGrid G;
    if (grid_of(shape, axisymmetric, 1.0, G)) return 0;
    return workspace_bytes(G);
}

int bssn_puncture_solve(const double* psi_bl, const double* curvature_squared, const int32_t shape[3], double dx,
                        int32_t axisymmetric, double newton_tolerance, int32_t max_newton_iterations,
                        double linear_tolerance, int32_t max_linear_iterations, double* u, double* psi,
                        double* residual_history, int32_t* history_length, int32_t* linear_iterations,
                        void* workspace, size_t workspace_bytes_, void* stream) {
    if (!psi_bl || !curvature_squared || !u || !psi || !residual_history || !history_length)
        return fail(BSSN_ERR_INVALID, "bssn_puncture_solve: null pointer");
    SolveGrid G;
    if (int e = grid_of(shape, axisymmetric, dx, G)) return e;
    if (!(newton_tolerance > 0.0) || !std::isfinite(newton_tolerance))
        return fail(BSSN_ERR_INVALID, "newton_tolerance must be finite and positive");
    if (!(linear_tolerance > 0.0) || !std::isfinite(linear_tolerance))
        return fail(BSSN_ERR_INVALID, "linear_tolerance must be finite and positive");
    if (max_newton_iterations < 0) return fail(BSSN_ERR_INVALID, "max_newton_iterations must be a nonnegative integer");
    if (max_linear_iterations < 1) return fail(BSSN_ERR_INVALID, "max_linear_iterations must be a positive integer");
    if (!workspace || workspace_bytes_ < workspace_bytes(G))
        return fail(BSSN_ERR_WORKSPACE, "workspace missing or smaller than bssn_puncture_workspace_bytes()");
    *history_length = 0;

    SolveStream* ss = nullptr;
    cudaError_t e = solve_stream(ss);
    if (e != cudaSuccess) return cuda_status(e, "bssn_puncture_solve");
    cudaStream_t caller = (cudaStream_t)stream;
    cudaStream_t s = ss->s;
    e = cudaEventRecord(ss->in, caller);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(s, ss->in, 0);
    if (e != cudaSuccess) return cuda_status(e, "bssn_puncture_solve");

    const long long n = G.size();
    const size_t vec_al = ((size_t)n * sizeof(double) + 255) & ~(size_t)255;
    char* base = static_cast<char*>(workspace);
    double* v[V_COUNT];
    for (int q = 0; q < V_COUNT; ++q) v[q] = reinterpret_cast<double*>(base + q * vec_al);
    double* partial = reinterpret_cast<double*>(base + V_COUNT * vec_al);
    const size_t pbytes = (size_t)max_blocks(G) * kMaxSums * sizeof(double);
    SolveCtrl* ctrl = reinterpret_cast<SolveCtrl*>(base + V_COUNT * vec_al + ((pbytes + 255) & ~(size_t)255));

    e = cudaMemsetAsync(base, 0, V_COUNT * vec_al, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(ctrl, 0, sizeof(SolveCtrl), s);
    if (e == cudaSuccess) e = cudaMemsetAsync(u, 0, (size_t)n * sizeof(double), s);
    if (e != cudaSuccess) return cuda_status(e, "bssn_puncture_solve");

    const unsigned ub = update_blocks(n);
    const unsigned cg_blocks = G.axi ? 0u : cg_apply_blocks(G);
    const dim3 axi_grid(G.axi ? (G.n[2] - 2 + kAz - 1) / kAz : 1, G.axi ? (G.n[0] - 1 + kAr - 1) / kAr : 1, 1);

    // one chunk of kChunk Krylov iterations (kChunk is even, so the ping-pong
    // buffers line up from chunk to chunk)
    int chunk_launches = 0;
    auto enqueue_chunk = [&]() {
        for (int j = 0; j < kChunk; ++j) {
            double* pin = v[j % 2 ? V_P1 : V_P0];
            double* pout = v[j % 2 ? V_P0 : V_P1];
            if (!G.axi) {
                BSSN_LAUNCH(KC_SOLVE_APPLY, k_cg_apply, cg_blocks, kTz * kTy, s, v[V_R], pin, pout, v[V_CENTRE],
                            v[V_Q], v[V_X], G, ctrl, partial);
                BSSN_LAUNCH(KC_SOLVE_UPDATE, k_cg_update, ub, kPunctThreads, s, v[V_R], v[V_Q], n, ctrl, partial);
                chunk_launches += 2;
            } else {
                // q ping-pongs as well: the p kernel reads the previous p and q around each cell
                double* qin = v[j % 2 ? V_Q1 : V_Q];
                double* qout = v[j % 2 ? V_Q : V_Q1];
                BSSN_LAUNCH(KC_SOLVE_APPLY, k_bicg_p, axi_grid, kAz * kAr, s, v[V_R], v[V_RHAT], pin, qin, pout, qout,
                            v[V_CENTRE], G, ctrl, partial);
                BSSN_LAUNCH(KC_SOLVE_APPLY, k_bicg_s, axi_grid, kAz * kAr, s, v[V_R], qout, v[V_S], v[V_T],
                            v[V_CENTRE], G, ctrl, partial);
                BSSN_LAUNCH(KC_SOLVE_UPDATE, k_bicg_x, ub, kPunctThreads, s, v[V_X], v[V_R], v[V_RHAT], pout, v[V_S],
                            v[V_T], n, ctrl, partial);
                chunk_launches += 3;
            }
        }
    };
    cudaGraphExec_t exec = nullptr;
    auto finish = [&](int code) {
        if (exec) cudaGraphExecDestroy(exec);
        cudaEventRecord(ss->out, s);
        cudaStreamWaitEvent(caller, ss->out, 0);
        return code;
    };
    // Replay the chunk as a CUDA graph unless per-kernel profiling is on
    // (which times every launch with events of its own).
    if (!profiling_enabled() && cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
        cudaGraph_t graph = nullptr;
        enqueue_chunk();
        count_launches(-chunk_launches);   // recorded, not run
        e = cudaStreamEndCapture(s, &graph);
        if (e == cudaSuccess) e = cudaGraphInstantiate(&exec, graph, 0);
        if (graph) cudaGraphDestroy(graph);
        if (e != cudaSuccess) {
            exec = nullptr;
            return finish(cuda_status(e, "bssn_puncture_solve (graph capture)"));
        }
    }
    auto run_chunk = [&]() -> cudaError_t {
        if (!exec) {
            chunk_launches = 0;
            enqueue_chunk();
            return cudaGetLastError();
        }
        count_launches(chunk_launches);
        return cudaGraphLaunch(exec, s);
    };

    const double tol2 = linear_tolerance * linear_tolerance;
    SolveCtrl host;
    int count = 0;
    for (int it = 0; it <= max_newton_iterations; ++it) {
        BSSN_LAUNCH(KC_SOLVE_NEWTON, k_newton_residual, ub, kPunctThreads, s, u, psi_bl, curvature_squared, G, v[V_R],
                    G.axi ? v[V_RHAT] : nullptr, v[V_CENTRE], partial, ctrl, tol2, max_linear_iterations,
                    G.axi ? 0 : 1);
        e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaMemcpyAsync(&host, ctrl, sizeof(SolveCtrl), cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) return finish(cuda_status(e, "bssn_puncture_solve"));
        if (G.axi && it > 0) {
            // checks of the previous correction (bowen_york_solver.py:471-474)
            if (host.bad_u) return finish(fail(BSSN_ERR_NONFINITE, "Newton-Raphson correction is nonfinite"));
            if (host.bad_psi)
                return finish(fail(BSSN_ERR_NONFINITE, "Newton-Raphson correction made psi nonpositive"));
        }
        residual_history[count++] = host.rms;
        *history_length = count;
        if (G.axi && !std::isfinite(host.rms))
            return finish(fail(BSSN_ERR_NONFINITE, "Newton-Raphson solve produced a nonfinite residual"));
        if (host.rms <= newton_tolerance) break;
        if (it == max_newton_iterations) {
            char msg[160];
            std::snprintf(msg, sizeof(msg), "Newton-Raphson solve did not converge: RMS residual %.3e exceeds %.3e.",
                          host.rms, newton_tolerance);
            return finish(fail(BSSN_ERR_NOT_CONVERGED, msg));
        }
        e = cudaMemsetAsync(v[V_X], 0, (size_t)n * sizeof(double), s);
        if (e != cudaSuccess) return finish(cuda_status(e, "bssn_puncture_solve"));
        bool done = host.done != 0;
        while (!done) {
            e = run_chunk();
            if (e == cudaSuccess) e = cudaMemcpyAsync(&host, ctrl, sizeof(SolveCtrl), cudaMemcpyDeviceToHost, s);
            if (e == cudaSuccess) e = cudaStreamSynchronize(s);
            if (e != cudaSuccess) return finish(cuda_status(e, "bssn_puncture_solve"));
            done = host.done != 0;
        }
        if (!G.axi && host.k > 0) {
            // iteration k - 1 wrote its p to P0 when odd, P1 when even
            const double* p_last = v[(host.k - 1) % 2 ? V_P0 : V_P1];
            BSSN_LAUNCH(KC_SOLVE_UPDATE, k_cg_finish, ub, kPunctThreads, s, v[V_X], p_last, n, ctrl);
        }
        if (linear_iterations) linear_iterations[it] = host.k;
        BSSN_LAUNCH(KC_SOLVE_UPDATE, k_newton_update, ub, kPunctThreads, s, u, v[V_X], n);
    }
    BSSN_LAUNCH(KC_SOLVE_UPDATE, k_psi_total, ub, kPunctThreads, s, psi_bl, u, psi, n);
    return finish(cuda_status(cudaGetLastError(), "bssn_puncture_solve"));
}

}  // extern "C"
