// BSSN right-hand side on a padded patch (sm_103a).
//
// One RHS evaluation is a short pipeline of point-parallel kernels over the
// compute box of a padded patch:
//   k_first_derivs   first derivatives of gt, W, alpha, beta (and, when
//                    kappa != 0, of At, K and B_i^j) on the compute box grown
//                    by the outer-stencil reach: the inner factors of every
//                    composed mixed second derivative D1(D1(f, inner), outer)
//                    (JAX_BSSN/bssn/geometry.py:47-56,93-99,
//                    JAX_BSSN/bssn/conformal_connection.py:115-137,
//                    JAX_BSSN/bssn/constraints.py:165-184)
//   k_rhs_gauge      dt gt_ij, dt W, dt alpha, dt beta^i
//                    (JAX_BSSN/bssn/spatial_metric.py:17-106, shift_and_lapse.py:65-132)
//   k_rhs_curv       FP64 form: dt K, dt Gt^i and dt At_ij in one pass
//                    (sharing the inverse metric, Christoffels, lapse Hessian)
//   k_rhs_kgt        FP32 form: dt K, dt Gt^i (JAX_BSSN/bssn/extrinsic_curvature.py:31-92,
//                    conformal_connection.py:19-162)
//   k_rhs_at         FP32 form: dt At_ij incl. W^2 R_ij, W^2 D_i D_j alpha
//                    (JAX_BSSN/bssn/extrinsic_curvature.py:119-224, geometry.py:21-186)
//   k_mom_*          kappa != 0 only: M_i, d_l M_i and the constraint-damping
//                    term (JAX_BSSN/bssn/constraints.py:22-213)
//   k_sommerfeld     radial Sommerfeld replacement on active owned faces
//                    (JAX_BSSN/evolution/boundaries.py:150-171)
// Operators commute along different axes, so each mixed derivative is formed
// once (outer axis = the larger index, as in the reference's upper triangle)
// and used for both orderings.  (The reference also forms the other ordering;
// on the second row from a Sommerfeld face that one applies the one-sided
// closure to O(1) samples, so its lower-triangle entries differ from the
// upper ones by that closure's rounding.)
//
// Two arithmetic forms share this source (template parameter R):
//   double  the plain FP64 form; kernels read the FP64 state directly.
//   float   the FP32-arithmetic form: k_perturb first writes the state as
//           float perturbations about a constant background (1 for the
//           conformal-metric diagonal, W and alpha; the state's own value at
//           the box's first sample for the shift and K, so a uniform shift or
//           a constant-K slice is removed too; 0 otherwise), so small
//           deviations keep float's relative precision through every
//           stencil; the algebra then runs in float.  W, alpha, the shift and
//           K enter the pointwise terms as full values read from the FP64
//           state, and 1/W
//           (large near punctures) is formed in FP64.  The RHS is written in
//           FP64, and the RK4 combination stays FP64.
#include <atomic>
#include <climits>
#include <cstdint>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include <cuda.h>

#include "bssn_fields.cuh"
#include "bssn_kernels.h"
#include "bssn_profile.h"

namespace bssn {

constexpr int kThreads = 128;
constexpr double kPi = 3.141592653589793;   // the double nearest pi (numpy.pi)

template <typename R>
constexpr bool kPerturbative = std::is_same<R, float>::value;

// Stencil numerators keep the reference's rounding, in the FP64 form, for the
// fields that can carry a constant background: the unit diagonal of gt, W and
// alpha, and the shift (a uniform shift is a constant background too).  Fields
// whose background is zero (At, K, Gt, the off-diagonal gt), and every field of
// the FP32 form (which stores perturbations), take the regrouped numerators.
template <typename R>
constexpr bool kExactBg = !kPerturbative<R>;

// Unrolling of the gauge kernel's per-component loops: the FP32 form is
// issue-bound there, and full unrolling turns runtime component indices into
// constants (the larger curvature kernels lose more to occupancy and
// instruction fetch than they gain); the FP64 form is bound by FP64
// instructions and keeps compact loops.
template <typename R>
constexpr int kUnroll = kPerturbative<R> ? 8 : 1;
__host__ __device__ constexpr bool unit_diagonal(int s) { return s == 0 || s == 3 || s == 5; }

// Resident blocks per SM asked of the FP32 curvature kernels: 8 blocks of 128
// caps them at 64 registers.  They are latency-bound on stencil loads, and the
// extra warps outweigh the spills (measured: the At kernel 14% and the K/Gt
// kernel 3% faster than at 96 and 80 registers; 7 or 9 blocks do less well).
template <typename R>
constexpr int kMinBlocks = kPerturbative<R> ? 8 : 1;

__host__ __device__ constexpr bool has_background(int c) {
    return c == GXX || c == GYY || c == GZZ || c == CW || c == CALPHA;
}
// FP32 form: components whose perturbation is taken about their own value at
// one sample of the state (a uniform shift, a constant-K slice).
__host__ __device__ constexpr bool state_background(int c) {
    return c == BX || c == BY || c == BZ || c == CK;
}

__device__ __forceinline__ bool in_range(const Axis& a, int i) { return i >= a.lo && i < a.hi; }

// Up to ten boxes covered by one launch; blockIdx.y selects the box.
struct BoxSet {
    Box b[10];
    int n;
};

// The point a thread works on.
struct PointCtx {
    int ix[3];
    long long p;
};

// Full value of component comp at the point of the R-typed state: the FP32
// form adds back the unit background of the metric diagonal, W and alpha
// (the shift and K, whose background is taken from the state, are read in
// FP64 by full_exact).
template <typename R>
__device__ __forceinline__ R full(const R* __restrict__ u, int comp, const Geo& G, const PointCtx& c) {
    R v = u[comp * G.cs + c.p];
    if constexpr (kPerturbative<R>) {
        if (has_background(comp)) v += R(1);
    }
    return v;
}

// W or alpha as a full value: from the FP64 state in the FP32 form (no
// background cancellation near a puncture), from u itself in the FP64 form.
template <typename R>
__device__ __forceinline__ R full_exact(const R* __restrict__ u, const double* __restrict__ u64, int c,
                                        long long cs, long long p) {
    if constexpr (kPerturbative<R>) return static_cast<R>(u64[c * cs + p]);
    else return u[c * cs + p];
}

// ---------------------------------------------------------------------------
// FP32 form: float perturbations of the state on a region
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kThreads)
k_perturb(const double* __restrict__ u, float* __restrict__ uf, Geo G, Box region, long long p0) {
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= box_threads(G, region)) return;
    const long long off = instance_offset(G, region, t);
    int ix[3];
    region.coords(t, ix);
    const long long p = lin(G, ix) + off, cs = G.cs;
    auto perturbation = [&](int c) {
        const double b = has_background(c) ? 1.0 : (state_background(c) ? u[c * cs + p0 + off] : 0.0);
        return u[c * cs + p] - b;
    };
#pragma unroll
    for (int c = 0; c < NCOMP; ++c) uf[c * cs + p] = static_cast<float>(perturbation(c));
    // Paired form: low words of the fields whose second derivatives are
    // taken.  hi + lo carries the perturbation to ~48 bits, so the 1/dx^2 of
    // D2 does not amplify the float rounding of the samples themselves.
    if (G.precision != kPrecisionF32Paired) return;
#pragma unroll
    for (int f = 0; f < NMIX; ++f) {
        const int c = mix_source(f);
        const double d = perturbation(c);
        uf[(NCOMP + f) * cs + p] = static_cast<float>(d - (double)static_cast<float>(d));
    }
}

// The low word of NMIX field f in the FP32 form's perturbation array.
__device__ __forceinline__ const float* low_word(const float* uf, const Geo& G, int f, long long p) {
    return uf + (NCOMP + f) * G.cs + p;
}

// ---------------------------------------------------------------------------
// inner first derivatives
// ---------------------------------------------------------------------------
template <typename R, bool Closed>
__global__ void __launch_bounds__(kThreads)
k_first_derivs(const R* __restrict__ u, const R* __restrict__ der, R* __restrict__ d1, Geo G, BoxSet S,
               int with_mom) {
    const Box& ext = S.b[blockIdx.y];
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= box_threads(G, ext)) return;
    const long long off = instance_offset(G, ext, t);
    int ix[3];
    if constexpr (Closed) ext.coords(t, ix);
    else ext.coords_z(t, ix);
    const long long p = lin(G, ix) + off;
    const long long cs = G.cs;
    const int nfield = with_mom ? NMIX + NMIX_MOM : NMIX;
#pragma unroll 1
    for (int d = 0; d < 3; ++d) {
        if (!in_range(G.ax[d], ix[d])) continue;
#pragma unroll 1
        for (int f = 0; f < NMIX; ++f) {
            R v = D1<R, Closed>(u + mix_source(f) * cs + p, G, d, ix[d]);
            if constexpr (kPerturbative<R>)
                if (G.precision == kPrecisionF32Paired) v += D1<R, Closed>(low_word(u, G, f, p), G, d, ix[d]);
            d1[((long long)(d * nfield + f)) * cs + p] = v;
        }
        if (with_mom) {
#pragma unroll 1
            for (int f = 0; f < 7; ++f)  // At (6), K
                d1[((long long)(d * nfield + NMIX + f)) * cs + p] = D1<R, Closed>(u + (AXX + f) * cs + p, G, d, ix[d]);
#pragma unroll 1
            for (int f = 0; f < 9; ++f)  // B_i^j from the derived buffer (slots 6..14)
                d1[((long long)(d * nfield + NMIX + 7 + f)) * cs + p] = D1<R, Closed>(der + (6 + f) * cs + p, G, d, ix[d]);
        }
    }
}

// AnyOrder = false: the box is known to run z fastest (closure-free interior boxes).
template <bool AnyOrder = true>
__device__ __forceinline__ bool point(const Box& B, PointCtx& c, const Geo& G) {
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= box_threads(G, B)) return false;
    const long long off = instance_offset(G, B, t);
    if constexpr (AnyOrder) B.coords(t, c.ix);
    else B.coords_z(t, c.ix);
    c.p = lin(G, c.ix) + off;
    return true;
}

// d1 buffer accessor: first derivative along d of stored field f.
template <typename R>
__device__ __forceinline__ const R* d1ptr(const R* d1, const Geo& G, int nfield, int d, int f, long long p) {
    return d1 + ((long long)(d * nfield + f)) * G.cs + p;
}

// Mixed second derivative d_m d_n of stored field f (m != n): outer axis is
// max(m,n), inner axis min(m,n).
template <typename R, bool Closed>
__device__ __forceinline__ R mixed(const R* d1, const Geo& G, int nfield, int f, int m, int n, const PointCtx& c) {
    const int inner = m < n ? m : n;
    const int outer = m < n ? n : m;
    return D1<R, Closed>(d1ptr(d1, G, nfield, inner, f, c.p), G, outer, c.ix[outer]);
}

// Symmetric Hessian of stored field f whose state component is comp:
// h[sym(i,j)] = d_i d_j f, D2 on the diagonal.
template <typename R, bool Closed, bool Exact = true>
__device__ __forceinline__ void hessian(const R* __restrict__ u, const R* d1, const Geo& G, int nfield, int comp,
                                        int f, const PointCtx& c, R (&h)[6]) {
    const R* fp = u + comp * G.cs + c.p;
    h[0] = D2<R, Closed, Exact>(fp, G, 0, c.ix[0]);
    h[3] = D2<R, Closed, Exact>(fp, G, 1, c.ix[1]);
    h[5] = D2<R, Closed, Exact>(fp, G, 2, c.ix[2]);
    if constexpr (kPerturbative<R>) {
        if (G.precision == kPrecisionF32Paired) {
            const float* lo = low_word(u, G, f, c.p);
            h[0] += D2<R, Closed, false>(lo, G, 0, c.ix[0]);
            h[3] += D2<R, Closed, false>(lo, G, 1, c.ix[1]);
            h[5] += D2<R, Closed, false>(lo, G, 2, c.ix[2]);
        }
    }
    h[1] = mixed<R, Closed>(d1, G, nfield, f, 0, 1, c);
    h[2] = mixed<R, Closed>(d1, G, nfield, f, 0, 2, c);
    h[4] = mixed<R, Closed>(d1, G, nfield, f, 1, 2, c);
}

template <typename R>
__device__ __forceinline__ R contract_sym(const R (&a)[6], const R (&b)[6]) {
    return a[0] * b[0] + a[3] * b[3] + a[5] * b[5] + R(2) * (a[1] * b[1] + a[2] * b[2] + a[4] * b[4]);
}

// W^2 D_i D_j alpha (JAX_BSSN/bssn/geometry.py:122-186)
template <typename R, bool Closed>
__device__ __forceinline__ void w2_lapse_hessian(const R* __restrict__ u, const R* d1, const Geo& G, int nfield,
                                                 const PointCtx& c, const R (&g)[6], const R (&gi)[6],
                                                 const R (&c2)[3][6], const R (&dW)[3], const R (&da)[3], R W,
                                                 R (&out)[6]) {
    R h[6];
    hessian<R, Closed, kExactBg<R>>(u, d1, G, nfield, CALPHA, MIX_ALPHA, c, h);
    R gw = R(0);  // gt^mn d_m W d_n alpha
#pragma unroll
    for (int n = 0; n < 3; ++n) gw += (gi[sym(0, n)] * dW[0] + gi[sym(1, n)] * dW[1] + gi[sym(2, n)] * dW[2]) * da[n];
    const R W2 = W * W;
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = i; j < 3; ++j) {
            const int s = sym(i, j);
            const R conf = h[s] - (c2[0][s] * da[0] + c2[1][s] * da[1] + c2[2][s] * da[2]);
            const R grad = dW[i] * da[j] + dW[j] * da[i] - g[s] * gw;
            out[s] = W2 * conf + W * grad;
        }
}

template <typename R>
__device__ __forceinline__ void load_sym(const R* __restrict__ u, int base, const Geo& G, const PointCtx& c,
                                         R (&v)[6]) {
#pragma unroll
    for (int s = 0; s < 6; ++s) v[s] = full(u, base + s, G, c);
}

template <typename R>
__device__ __forceinline__ void load_metric_derivs(const R* d1, const Geo& G, int nfield, long long p,
                                                   R (&dg)[3][6]) {
#pragma unroll
    for (int k = 0; k < 3; ++k)
#pragma unroll
        for (int s = 0; s < 6; ++s) dg[k][s] = d1ptr(d1, G, nfield, k, MIX_G + s, p)[0];
}

// W^2 R_ij without inverse powers of W (JAX_BSSN/bssn/geometry.py:21-119).
template <typename R, bool Closed>
__device__ __forceinline__ void w2_ricci(const R* __restrict__ u, const R* d1, const Geo& G, int nfield,
                                         const PointCtx& c, const R (&g)[6], const R (&gi)[6], const R (&c1)[3][6],
                                         const R (&c2)[3][6], const R (&dW)[3], R W, R (&w2r)[6]) {
    const long long cs = G.cs, p = c.p;
    // The FP64 form is bound by FP64 instructions, not loads: it re-reads the
    // metric derivatives d_m gt_ij and uses d_m gt_jk = Gamma_jkm + Gamma_kjm,
    // which needs fewer operations than the Christoffel sums.
    constexpr bool reload = !kPerturbative<R>;
    auto dgm = [&](int m, int s) { return d1ptr(d1, G, nfield, m, MIX_G + s, p)[0]; };
    // --- conformal Ricci tensor (geometry.py:44-81) ---
    R ric[6];
    {
        // -1/2 gt^mn with the off-diagonal entries doubled: -1/2 gt^mn d_m d_n gt_ij
        // as a six-term sum over the symmetric Hessian
        const R hg[6] = {R(-0.5) * gi[0], -gi[1], -gi[2], R(-0.5) * gi[3], -gi[4], R(-0.5) * gi[5]};
#pragma unroll 1
        for (int s = 0; s < 6; ++s) {
            R h[6];
            if (unit_diagonal(s)) hessian<R, Closed, kExactBg<R>>(u, d1, G, nfield, GXX + s, MIX_G + s, c, h);
            else hessian<R, Closed, false>(u, d1, G, nfield, GXX + s, MIX_G + s, c, h);
            ric[s] = hg[0] * h[0] + hg[1] * h[1] + hg[2] * h[2] + hg[3] * h[3] + hg[4] * h[4] + hg[5] * h[5];
        }
    }
    {
        const R Gt[3] = {full(u, GTX, G, c), full(u, GTY, G, c), full(u, GTZ, G, c)};
        R dG[3][3];  // dG[d][i] = d_d Gt^i
#pragma unroll 1
        for (int d = 0; d < 3; ++d)
#pragma unroll 1
            for (int i = 0; i < 3; ++i) dG[d][i] = D1<R, Closed>(u + (GTX + i) * cs + p, G, d, c.ix[d]);
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int j = i; j < 3; ++j) {
                R t2 = R(0), t3 = R(0);  // t3 = Gt^m (Gamma_ijm + Gamma_jim) = Gt^m d_m gt_ij
#pragma unroll
                for (int m = 0; m < 3; ++m) {
                    t2 += g[sym(m, i)] * dG[j][m] + g[sym(m, j)] * dG[i][m];
                    if constexpr (reload) t3 += Gt[m] * dgm(m, sym(i, j));
                    else t3 += Gt[m] * (c1[i][sym(j, m)] + c1[j][sym(i, m)]);
                }
                ric[sym(i, j)] += R(0.5) * (t2 + t3);
            }
    }
    // term4 + term5, one k at a time to bound live registers.  Both contract
    // X[n][i] = g^mn Gamma^k_mi:
    //   term4 = X[n][i] Gamma_jkn + X[n][j] Gamma_ikn,  term5 = X[n][i] Gamma_kjn
    // (term5 = Gamma^k_im g^mn Gamma_kjn with the symmetric Gamma^k_mi).
#pragma unroll 1
    for (int kk = 0; kk < 3; ++kk) {
        R X[3][3];
#pragma unroll
        for (int a = 0; a < 3; ++a)
#pragma unroll
            for (int b = 0; b < 3; ++b)
                X[a][b] = gi[sym(0, a)] * c2[kk][sym(0, b)] + gi[sym(1, a)] * c2[kk][sym(1, b)]
                          + gi[sym(2, a)] * c2[kk][sym(2, b)];
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int j = i; j < 3; ++j) {
                R acc = ric[sym(i, j)];
#pragma unroll
                for (int n = 0; n < 3; ++n) {
                    if constexpr (reload) acc += X[n][i] * dgm(n, sym(j, kk)) + X[n][j] * c1[i][sym(kk, n)];
                    else acc += X[n][i] * (c1[j][sym(kk, n)] + c1[kk][sym(j, n)]) + X[n][j] * c1[i][sym(kk, n)];
                }
                ric[sym(i, j)] = acc;
            }
    }
    // --- W terms: W (D_i D_j W + gt_ij lap W) - 2 gt_ij |dW|^2 (geometry.py:84-117) ---
    {
        R hW[6];
        hessian<R, Closed, kExactBg<R>>(u, d1, G, nfield, CW, MIX_W, c, hW);
#pragma unroll
        for (int s = 0; s < 6; ++s) hW[s] -= c2[0][s] * dW[0] + c2[1][s] * dW[1] + c2[2][s] * dW[2];
        const R lap = contract_sym(gi, hW);
        R grad2 = R(0);  // gt^mn d_m W d_n W
#pragma unroll
        for (int n = 0; n < 3; ++n)
            grad2 += (gi[sym(0, n)] * dW[0] + gi[sym(1, n)] * dW[1] + gi[sym(2, n)] * dW[2]) * dW[n];
        const R W2 = W * W;
#pragma unroll
        for (int s = 0; s < 6; ++s) w2r[s] = W2 * ric[s] + (W * (hW[s] + g[s] * lap) - R(2) * g[s] * grad2);
    }
}

// ---------------------------------------------------------------------------
// dt gt_ij, dt W, dt alpha, dt beta^i
// ---------------------------------------------------------------------------
template <typename R, bool Closed>
__global__ void __launch_bounds__(kThreads)
k_rhs_gauge(const R* __restrict__ u, const double* __restrict__ u64, const R* __restrict__ d1,
            double* __restrict__ k, Geo G, BoxSet S, int nfield) {
    PointCtx c;
    if (!point<Closed>(S.b[blockIdx.y], c, G)) return;
    const long long cs = G.cs, p = c.p;
    const R beta[3] = {full_exact(u, u64, BX, cs, p), full_exact(u, u64, BY, cs, p), full_exact(u, u64, BZ, cs, p)};
    R bs[3];
    shift_over_12dx(G, beta, bs);
    R db[3][3];  // db[i][j] = d_j beta^i
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) db[i][j] = d1ptr(d1, G, nfield, j, MIX_B + i, p)[0];
    const R div = db[0][0] + db[1][1] + db[2][2];
    const R alpha = full_exact(u, u64, CALPHA, cs, p);
    const R K = full_exact(u, u64, CK, cs, p);
    const R W = full_exact(u, u64, CW, cs, p);
    R g[6];
    load_sym(u, GXX, G, c, g);

    R P[6];  // pointwise terms: Lie terms - 2/3 gt_ij div beta - 2 alpha At_ij
    {
        const R m23div = R(-2.0 / 3.0) * div, m2a = R(-2.0) * alpha;
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int j = i; j < 3; ++j) {
                R lie = R(0);
#pragma unroll
                for (int m = 0; m < 3; ++m) lie += g[sym(m, i)] * db[m][j] + g[sym(m, j)] * db[m][i];
                const int s = sym(i, j);
                P[s] = lie + m23div * g[s] + m2a * full(u, AXX + s, G, c);
            }
    }
#pragma unroll (kUnroll<R>)
    for (int s = 0; s < 6; ++s) {
        const R* f = u + (GXX + s) * cs + p;
        R v;
        if (unit_diagonal(s))
            v = (ADV<R, Closed, kExactBg<R>>(f, G, c.ix, beta, bs) + P[s]) + KO<R, Closed, kExactBg<R>>(f, G, c.ix);
        else
            v = (ADV<R, Closed, false>(f, G, c.ix, beta, bs) + P[s]) + KO<R, Closed, false>(f, G, c.ix);
        k[(GXX + s) * cs + p] = v;
    }
    {
        const R* f = u + CW * cs + p;
        const R v = ADV<R, Closed, kExactBg<R>>(f, G, c.ix, beta, bs) + R(1.0 / 3.0) * alpha * W * K
                    - R(1.0 / 3.0) * W * div;
        k[CW * cs + p] = v + KO<R, Closed, kExactBg<R>>(f, G, c.ix);
    }
    {
        const R* f = u + CALPHA * cs + p;
        const R slicing = (G.gauge == 0) ? -(alpha * alpha) * K : R(-2.0) * alpha * K;
        k[CALPHA * cs + p] = slicing + ADV<R, Closed, kExactBg<R>>(f, G, c.ix, beta, bs)
                             + KO<R, Closed, kExactBg<R>>(f, G, c.ix);
    }
#pragma unroll (kUnroll<R>)
    for (int i = 0; i < 3; ++i) {
        const R* f = u + (BX + i) * cs + p;
        R v;
        if (G.zero_shift) {
            v = R(0) * beta[i];
        } else {
            v = BSSN_CO(R, G, g) * full(u, GTX + i, G, c) + ADV<R, Closed, kExactBg<R>>(f, G, c.ix, beta, bs)
                + (-BSSN_CO(R, G, eta)) * beta[i];
            v = v + KO<R, Closed, kExactBg<R>>(f, G, c.ix);
        }
        k[(BX + i) * cs + p] = v;
    }
}

// ---------------------------------------------------------------------------
// FP32 forms: shared pieces of the TMA-staged interior kernels.  Each stages
// halo boxes of the float state (or of its stored first derivatives) in
// shared memory with cp.async.bulk.tensor loads that complete on mbarriers;
// every wait is bounded, and a CTA whose wait gives up counts a timeout,
// waits once more (bounded) for its copies in flight and leaves its samples
// unwritten.
// ---------------------------------------------------------------------------
namespace tma {
constexpr int TZ = 32, TY = 8, TX = 4;                   // first-derivative tile
constexpr int THREADS = 256;                             // four z samples per thread
constexpr long long kWaitLimit = 1LL << 24;              // try_wait polls before giving up
static_assert(TX * TY * (TZ / 4) == THREADS, "one thread per four z samples");

__device__ __forceinline__ unsigned smem_addr(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }
// A global load the compiler may not merge with an earlier load of the same
// address: re-reading a value (an L1 hit) instead of holding it in a register
// across a phase that would spill.
__device__ __forceinline__ float reload(const float* q) {
    float v;
    asm volatile("ld.global.nc.f32 %0, [%1];" : "=f"(v) : "l"(q));
    return v;
}

__device__ __forceinline__ void bar_init(unsigned long long* bar) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(bar)) : "memory");
}
// Bounded wait on a tile's mbarrier phase; false when it gave up.
__device__ __forceinline__ bool bar_wait(unsigned long long* bar, unsigned phase) {
    for (long long i = 0; i < kWaitLimit; ++i) {
        unsigned done;
        asm volatile(
            "{ .reg .pred p; mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2; selp.u32 %0, 1, 0, p; }"
            : "=r"(done) : "r"(smem_addr(bar)), "r"(phase) : "memory");
        if (done) return true;
    }
    return false;
}

// Upwind numerator (units of 1/(12 dx)) from a 7-tap window a[k + 3] = f(+k),
// the side chosen by c (the generic kernel's up1_num_fused).
__device__ __forceinline__ float up1(const float (&a)[7], float c) {
    if (c > 0.0f) return (((-3.0f * a[2] + -10.0f * a[3]) + 18.0f * a[4]) + -6.0f * a[5]) + a[6];
    return (((-a[0] + 6.0f * a[1]) + -18.0f * a[2]) + 10.0f * a[3]) + 3.0f * a[4];
}
// Sixth-difference numerator from differences to the centre (ko_num_pairs).
__device__ __forceinline__ float ko(const float (&a)[7]) {
    const float f0 = a[3];
    const float s1 = (a[4] - f0) + (a[2] - f0), s2 = (a[5] - f0) + (a[1] - f0), s3 = (a[6] - f0) + (a[0] - f0);
    return (s3 - 6.0f * s2) + 15.0f * s1;
}
__device__ __forceinline__ float4 ld4(const float* p) { return *reinterpret_cast<const float4*>(p); }
__device__ __forceinline__ float at(const float4& v, int j) { return j == 0 ? v.x : (j == 1 ? v.y : (j == 2 ? v.z : v.w)); }
}  // namespace tma

// ---------------------------------------------------------------------------
// FP32 forms, first derivatives of the NMIX fields from TMA tiles: 32 x 8 x 4
// tiles with four z samples per thread, halo 2 in x and y (4 in z for the
// 16-byte rule), a three-deep ring of 40 x 12 x 8 boxes.  The paired form
// streams each field's low word too (the low words follow the 21
// perturbations, so one tensor map of 32 components covers both).  No MAD
// axis, kappa = 0.  Either the closure-free interior, or (where every closed
// axis is Sommerfeld at both ends) the whole box with the two D1 closure rows
// next to each face, face planes included.
// ---------------------------------------------------------------------------
namespace tma {
constexpr int DHZ = TZ + 8, DHY = TY + 4, DHX = TX + 4;        // 40 x 12 x 8
constexpr int DSY = DHZ, DSX = DHZ * DHY;
constexpr int DFIELD = DHZ * DHY * DHX;                        // 3840 floats
constexpr unsigned DFIELD_BYTES = DFIELD * 4;                  // 15360 (a multiple of 128)
constexpr int DNBUF = 3;
constexpr size_t DSMEM = (size_t)DNBUF * DFIELD_BYTES + DNBUF * sizeof(unsigned long long);
static_assert(DFIELD_BYTES % 128 == 0, "tile buffers must stay 128-byte aligned");

// Closure rows of D1 (the forward's d1_closed): code +1 / -1 the lower / upper
// face plane, +2 / -2 the row next to it, 0 elsewhere; the upper face first.
__device__ __forceinline__ int d1_code(const Axis& A, int c) {
    if (A.rbc) {
        const int r = A.end - 1 - c;
        if (r == 0 || r == 1) return -(r + 1);
    }
    if (A.lbc) {
        const int r = c - A.start;
        if (r == 0 || r == 1) return r + 1;
    }
    return 0;
}
// D1 on a closure row from its taps counted inward from the face (f1..f4 at
// 1..4 samples inward, fb one sample outward, on the row next to the face
// only), in difference form: rows 0 {-25/12, 4, -3, 4/3, -1/4} at 0..4 and 1
// {-1/4, -5/6, 3/2, -1/2, 1/12} at -1..3; an upper face mirrors them.
__device__ __forceinline__ float d1_closure(int code, float f0, float f1, float f2, float f3, float fx,
                                            float inv_dx) {
    const bool face = code == 1 || code == -1;   // fx is f4 on the face plane, fb on the next row
    const float v = face ? ((4.0f * (f1 - f0) + -3.0f * (f2 - f0)) + (4.0f / 3.0f) * (f3 - f0)) + -0.25f * (fx - f0)
                         : ((-0.25f * (fx - f0) + 1.5f * (f1 - f0)) + -0.5f * (f2 - f0)) + (1.0f / 12.0f) * (f3 - f0);
    return (code > 0 ? v : -v) * inv_dx;
}
// Box origin along x or y of a first-derivative tile starting at t0 (T
// samples): halo 2, lowered in a tile that holds an upper-face closure row so
// that the face plane's D1 reaches 4 below it (the box of 4 + T samples still
// covers every valid sample's taps above).
__device__ __forceinline__ int d1_origin(const Axis& A, int t0, int T, int blo, int bhi) {
    if (!A.rbc) return -2;
    const int xf = A.end - 1;
    const int lo = max(t0, max(xf - 1, blo)), hi = min(t0 + T - 1, min(xf, bhi - 1));
    return lo <= hi ? min(-2, xf - 4 - t0) : -2;
}

__device__ __forceinline__ void load_box(float* dst, const CUtensorMap* map, int z, int y, int x, int inst, int comp,
                                         unsigned long long* bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
    asm volatile(
        "cp.async.bulk.tensor.5d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5, %6}], [%7];"
        ::"r"(smem_addr(dst)), "l"(map), "r"(z), "r"(y), "r"(x), "r"(inst), "r"(comp), "r"(smem_addr(bar))
        : "memory");
}
}  // namespace tma

// Closed: the box may hold the two D1 closure rows next to Sommerfeld faces
// (their one-sided rows, the face planes included; box origins lowered at the
// upper faces); else it is closure-free.
template <bool Closed>
__global__ void __launch_bounds__(tma::THREADS)
k_first_derivs_tma(const __grid_constant__ CUtensorMap map, float* __restrict__ d1, Geo G, Box B, int z_base,
                   int tiles_z, int tiles_y, int nfield, int paired, int* __restrict__ timeouts) {
    using namespace tma;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    float* ring = reinterpret_cast<float*>(smem_raw);
    unsigned long long* bars = reinterpret_cast<unsigned long long*>(ring + DNBUF * DFIELD);
    const int tile = blockIdx.x, inst = blockIdx.y;
    const int z0 = z_base + TZ * (tile % tiles_z);
    const int y0 = B.lo[1] + TY * ((tile / tiles_z) % tiles_y);
    const int x0 = B.lo[0] + TX * (tile / (tiles_z * tiles_y));
    const int t = threadIdx.x;
    const int tz4 = t & 7, ty = (t >> 3) & 7, tx = t >> 6;
    const int x = x0 + tx, y = y0 + ty, zq = z0 + 4 * tz4;
    const bool col = x >= B.lo[0] && x < B.lo[0] + B.n[0] && y >= B.lo[1] && y < B.lo[1] + B.n[1];
    // box origins in x and y; a column outside the box reads as if at the
    // tile origin (a lowered box ends below it)
    const int ox = Closed ? d1_origin(G.ax[0], x0, TX, B.lo[0], B.lo[0] + B.n[0]) : -2;
    const int oy = Closed ? d1_origin(G.ax[1], y0, TY, B.lo[1], B.lo[1] + B.n[1]) : -2;
    const int rx = Closed && !col ? 0 : tx, ry = Closed && !col ? 0 : ty;
    int code[3][4];   // D1 closure rows (x and y per column, z per sample)
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        code[0][j] = Closed && col ? d1_code(G.ax[0], x) : 0;
        code[1][j] = Closed && col ? d1_code(G.ax[1], y) : 0;
        code[2][j] = Closed && col ? d1_code(G.ax[2], zq + j) : 0;
    }
    // as the generic kernel: the derivative along an axis only where the
    // sample lies in that axis' compute range (not in the grown box's ghosts)
    bool write[3][4];
    bool all[3];
#pragma unroll
    for (int dd = 0; dd < 3; ++dd) all[dd] = true;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const bool v = col && zq + j >= B.lo[2] && zq + j < B.lo[2] + B.n[2];
        const int c3[3] = {x, y, zq + j};
#pragma unroll
        for (int dd = 0; dd < 3; ++dd) {
            write[dd][j] = v && c3[dd] >= G.ax[dd].lo && c3[dd] < G.ax[dd].hi;
            all[dd] = all[dd] && write[dd][j];
        }
    }
    // tiles: field f's value, then (paired) its low word
    const int ntile = paired ? 2 * NMIX : NMIX;
    auto comp_of = [&](int i) { return paired ? ((i & 1) ? NCOMP + (i >> 1) : mix_source(i >> 1)) : mix_source(i); };
    if (t == 0) {
        for (int b = 0; b < DNBUF; ++b) bar_init(&bars[b]);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    __syncthreads();
    if (t == 0)
        for (int i = 0; i < DNBUF && i < ntile; ++i)
            load_box(ring + i * DFIELD, &map, z0 - 4, y0 + oy, x0 + ox, inst, comp_of(i), &bars[i], DFIELD_BYTES);
    const long long cs = G.cs;
    const long long p0 = ((long long)x * G.ax[1].P + y) * G.ax[2].P + zq + (long long)inst * G.istride;
    const int base = ((rx - ox) * DHY + (ry - oy)) * DHZ + 4 + 4 * tz4;
    const float a1 = G.gf.d1a, a2 = G.gf.d1b, inv_dx = G.gf.inv_dx;
    bool closure_x = false, closure_y = false, closure_z = false;
#pragma unroll
    for (int j = 0; j < 4; ++j) closure_z = closure_z || code[2][j] != 0;
    closure_x = code[0][0] != 0;
    closure_y = code[1][0] != 0;
    float acc[3][4];
    for (int i = 0; i < ntile; ++i) {
        const int b = i % DNBUF;
        const int missing = !bar_wait(&bars[b], (unsigned)((i / DNBUF) & 1));
        if (__syncthreads_or(missing)) {
            if (t == 0) {
                atomicAdd(timeouts, 1);
                for (int g = i; g < i + DNBUF && g < ntile; ++g) bar_wait(&bars[g % DNBUF], (unsigned)((g / DNBUF) & 1));
            }
            return;
        }
        const float* s = ring + b * DFIELD + base;
        float d[3][4];
        {   // z: a 12-sample window
            const float4 m = ld4(s - 4), c = ld4(s), q = ld4(s + 4);
            const float w[12] = {m.x, m.y, m.z, m.w, c.x, c.y, c.z, c.w, q.x, q.y, q.z, q.w};
#pragma unroll
            for (int j = 0; j < 4; ++j) d[2][j] = (w[5 + j] - w[3 + j]) * a1 + (w[6 + j] - w[2 + j]) * a2;
            if (Closed && closure_z) {
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    const int c = code[2][j];
                    if (c == 0) continue;
                    const bool up = c < 0, face = c == 1 || c == -1;
                    // taps inward from the face, from the 12-sample window
                    const float f0 = w[4 + j];
                    const float f1 = up ? w[3 + j] : w[5 + j], f2 = up ? w[2 + j] : w[6 + j];
                    const float f3 = up ? w[1 + j] : w[7 + j];
                    const float fx = face ? (up ? w[j] : w[8 + j]) : (up ? w[5 + j] : w[3 + j]);
                    d[2][j] = d1_closure(c, f0, f1, f2, f3, fx, inv_dx);
                }
            }
        }
#pragma unroll
        for (int dd = 0; dd < 2; ++dd) {   // x (0), y (1)
            const int st = dd == 0 ? DSX : DSY;
            const int c = code[dd][0];
            if (Closed && (dd == 0 ? closure_x : closure_y)) {
                // a column on a closure row: its taps inward from the face
                const int sg = c > 0 ? st : -st;
                const bool face = c == 1 || c == -1;
                const float4 f0 = ld4(s), f1 = ld4(s + sg), f2 = ld4(s + 2 * sg), f3 = ld4(s + 3 * sg);
                const float4 fx = ld4(s + (face ? 4 * sg : -sg));
#pragma unroll
                for (int j = 0; j < 4; ++j)
                    d[dd][j] = d1_closure(c, at(f0, j), at(f1, j), at(f2, j), at(f3, j), at(fx, j), inv_dx);
                continue;
            }
            const float4 m2 = ld4(s - 2 * st), m1 = ld4(s - st), p1 = ld4(s + st), p2 = ld4(s + 2 * st);
#pragma unroll
            for (int j = 0; j < 4; ++j) d[dd][j] = (at(p1, j) - at(m1, j)) * a1 + (at(p2, j) - at(m2, j)) * a2;
        }
        const bool lo_word = paired && (i & 1);
#pragma unroll
        for (int dd = 0; dd < 3; ++dd)
#pragma unroll
            for (int j = 0; j < 4; ++j) acc[dd][j] = lo_word ? acc[dd][j] + d[dd][j] : d[dd][j];
        if (!paired || lo_word) {
            const int f = paired ? (i >> 1) : i;
#pragma unroll
            for (int dd = 0; dd < 3; ++dd) {
                float* out = d1 + ((long long)(dd * nfield + f)) * cs + p0;
                if (all[dd]) {
                    *reinterpret_cast<float4*>(out) = make_float4(acc[dd][0], acc[dd][1], acc[dd][2], acc[dd][3]);
                } else {
#pragma unroll
                    for (int j = 0; j < 4; ++j)
                        if (write[dd][j]) out[j] = acc[dd][j];
                }
            }
        }
        __syncthreads();   // every thread is done with tile b
        if (t == 0 && i + DNBUF < ntile) {
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            load_box(ring + b * DFIELD, &map, z0 - 4, y0 + oy, x0 + ox, inst, comp_of(i + DNBUF), &bars[b],
                     DFIELD_BYTES);
        }
    }
}

// ---------------------------------------------------------------------------
// FP32 forms, interior curvature and gauge RHS from TMA boxes.  The generic
// float kernels k_rhs_at, k_rhs_kgt and k_rhs_gauge spend their issue slots
// on the address arithmetic and latency of several hundred scalar stencil
// taps per point.
// Here a CTA of 512 threads owns a 32 (z) x 4 (y) x 4 (x) tile, one sample
// per thread, and streams every stencilled input through a three-deep ring
// of shared-memory boxes, each one cp.async.bulk.tensor load completing on an
// mbarrier (three slots: two cost the loads' latency, four or a six-deep ring
// released in pairs crowd out the RHS kernels beside them):
//   a field's Hessian  value box, halo 2: the pure second derivatives (the
//                      paired form adds its low word's from a second box);
//                      boxes of its stored first derivatives along x and y,
//                      halo 2 along the outer axis only: d_y d_x, d_z d_x and
//                      d_z d_y;
//   Gt^i (dt At)       value box, halo 2: its first derivatives;
//   At_ij, K, Gt^i,    value box, halo 3: upwind advection and dissipation
//   gt, W, alpha, beta (and K's first derivatives).
// The RHS is linear in every one of these, so each box is folded into a few
// accumulators as soon as it is read; the pointwise terms are formed from
// single-sample reads while the first boxes load, and wait in registers
// (gauge) or shared memory (curvature).  With Sommerfeld faces closed at both
// ends of every closed axis the kernels also take the two rows next to each
// face, with the forward's one-sided rows (d1_row, d2_row, ko_row) and box
// origins lowered at the upper faces; the face planes stay the radial
// condition's.  Same terms as the generic kernels (no MAD axis; the curvature
// RHS for kappa = 0 in vacuum), regrouped.
// ---------------------------------------------------------------------------
namespace tma {
constexpr int AZ = 32, AY = 4, AX = 4;                    // tile; one sample per thread
constexpr int A_THREADS = AZ * AY * AX;                   // 512
constexpr int AHZ = AZ + 8;                               // z halo 4 keeps the origin on 16 bytes
constexpr int ANBUF = 3;
enum CurvBox { kBoxV2 = 0, kBoxDX = 1, kBoxDY = 2, kBoxV3 = 3 };
__host__ __device__ constexpr int a_hy(int kind) { return kind == kBoxV3 ? AY + 6 : (kind == kBoxDY ? AY : AY + 4); }
__host__ __device__ constexpr int a_hx(int kind) { return kind == kBoxV3 ? AX + 6 : (kind == kBoxV2 ? AX + 4 : AX); }
__host__ __device__ constexpr unsigned a_bytes(int kind) { return 4u * AHZ * a_hy(kind) * a_hx(kind); }
constexpr unsigned A_SLOT = a_bytes(kBoxV3);              // 16000 bytes, the largest box
// the ring, nq pointwise terms per sample, the ring's barriers
__host__ __device__ constexpr size_t curv_smem(int nq) {
    return (size_t)ANBUF * A_SLOT + (size_t)nq * A_THREADS * 4 + ANBUF * sizeof(unsigned long long);
}
constexpr int AT_NQ = 6, KGT_NQ = 4;
static_assert(A_SLOT % 128 == 0, "ring slots must stay 128-byte aligned");
static_assert(a_bytes(kBoxV2) % 16 == 0 && a_bytes(kBoxDX) % 16 == 0 && a_bytes(kBoxDY) % 16 == 0,
              "box sizes are multiples of 16 bytes");
// The boxes' tensor maps, by CurvBox: the FP32 state (components 0..NCOMP-1
// and the low words after them) with halo 2 and 3, and the first-derivative
// buffer with the d_x and the d_y box.
struct CurvMaps {
    CUtensorMap map[4];
};
struct CurvTile {
    int kind, comp;
};
// Box r of the Hessian group of stored field f: the value box, (paired) the
// low word's, the d_x box, the d_y box.
__device__ __forceinline__ CurvTile hessian_tile(int f, int r, int paired, int nfield) {
    if (r == 0) return {kBoxV2, mix_source(f)};
    if (paired && r == 1) return {kBoxV2, NCOMP + f};
    return (r - paired == 1) ? CurvTile{kBoxDX, f} : CurvTile{kBoxDY, nfield + f};
}
enum CurvSeq { kSeqAt = 0, kSeqKgt = 1, kSeqGauge = 2 };
__host__ __device__ constexpr int seq_tiles(int seq, int paired) {
    return seq == kSeqAt ? 33 + 8 * paired : (seq == kSeqKgt ? 16 + 4 * paired : NMIX);
}
// Box i of a kernel's fixed sequence.
//   dt At:       Hessian groups of gt_ij, W and alpha (stored fields 0..7),
//                the three Gt^i value boxes, the six At_ij halo-3 boxes;
//   dt K, Gt^i:  Hessian groups of alpha and beta^i (stored fields 7..10),
//                K's and the three Gt^i's halo-3 boxes;
//   gauge:       the halo-3 boxes of gt_ij, W, alpha and beta^i.
template <int Seq>
__device__ __forceinline__ CurvTile seq_tile(int i, int paired, int nfield) {
    const int gsz = 3 + paired;
    if constexpr (Seq == kSeqAt) {
        if (i < 8 * gsz) return hessian_tile(i / gsz, i % gsz, paired, nfield);
        i -= 8 * gsz;
        if (i < 3) return {kBoxV2, GTX + i};
        return {kBoxV3, AXX + (i - 3)};
    } else if constexpr (Seq == kSeqKgt) {
        if (i < 4 * gsz) return hessian_tile(MIX_ALPHA + i / gsz, i % gsz, paired, nfield);
        i -= 4 * gsz;
        return {kBoxV3, i == 0 ? CK : GTX + (i - 1)};
    } else {
        return {kBoxV3, mix_source(i)};
    }
}
// Fourth-order centred numerators from a shared-memory box at compile-time strides.
__device__ __forceinline__ float d2_box(const float* s, int st) {   // units of 1/(12 dx^2)
    const float f0 = s[0];
    return 16.0f * ((s[st] - f0) + (s[-st] - f0)) - ((s[2 * st] - f0) + (s[-2 * st] - f0));
}
__device__ __forceinline__ float d1_box(const float* s, int st, float a1, float a2) {
    return (s[st] - s[-st]) * a1 + (s[2 * st] - s[-2 * st]) * a2;
}
// Rows next to a Sommerfeld face, by row code: +1 / +2 the second / third
// sample from the lower face, -1 / -2 from the upper one, 0 elsewhere (the
// face plane itself is the radial condition's).  As the forward's float
// closures: one-sided D1 and D2 on rows 1, one-sided sixth differences on
// rows 1-2, in differences to the centre (each row's weights sum to zero);
// the upper face mirrors the lower (D1 changes sign).  The centred taps are
// read by every sample first, so in a warp that mixes rows only the one-sided
// rows' outer taps and sums diverge.
__device__ __forceinline__ float d1_row(const float* s, int st, int code, float a1, float a2, float inv_dx) {
    const float m2 = s[-2 * st], m1 = s[-st], p1 = s[st], p2 = s[2 * st];
    if (code == 1 || code == -1) {   // {-1/4, -5/6, 3/2, -1/2, 1/12} at -1..3
        const float f0 = s[0];
        const float b1 = code > 0 ? m1 : p1, f1 = code > 0 ? p1 : m1, f2 = code > 0 ? p2 : m2;
        const float f3 = s[3 * code * st];
        const float v = ((-0.25f * (b1 - f0) + 1.5f * (f1 - f0)) + -0.5f * (f2 - f0)) + (1.0f / 12.0f) * (f3 - f0);
        return (code > 0 ? v : -v) * inv_dx;
    }
    return (p1 - m1) * a1 + (p2 - m2) * a2;
}
__device__ __forceinline__ float d2_row(const float* s, int st, int code, float i12, float inv_dx2) {
    const float f0 = s[0], m2 = s[-2 * st], m1 = s[-st], p1 = s[st], p2 = s[2 * st];
    if (code == 1 || code == -1) {   // {5/6, -5/4, -1/3, 7/6, -1/2, 1/12} at -1..4
        const float b1 = code > 0 ? m1 : p1, f1 = code > 0 ? p1 : m1, f2 = code > 0 ? p2 : m2;
        const float f3 = s[3 * code * st], f4 = s[4 * code * st];
        const float v = ((5.0f / 6.0f) * (b1 - f0) + (-1.0f / 3.0f) * (f1 - f0))
                        + ((7.0f / 6.0f) * (f2 - f0) + -0.5f * (f3 - f0)) + (1.0f / 12.0f) * (f4 - f0);
        return v * inv_dx2;
    }
    return (16.0f * ((p1 - f0) + (m1 - f0)) - ((p2 - f0) + (m2 - f0))) * i12;
}
// Sixth-difference numerator on rows +-1 ({3, -20, 57, -90, 85, -48, 15, -2}
// at -1..6) and +-2 ({2, -13, 36, -55, 50, -27, 8, -1} at -2..5), from the
// centred window a[k + 3] = f(k) and the taps beyond it.
__device__ __forceinline__ float ko_row(const float (&a)[7], const float* s, int st, int code) {
    const bool up = code > 0;
    const int sg = up ? 1 : -1;
    const float f0 = a[3];
    // w(o) = f(sg o) - f0 for |o| <= 3, with compile-time window indices
    auto w = [&](int o) {
        const float lo = o == -2 ? a[1] : (o == -1 ? a[2] : (o == 1 ? a[4] : (o == 2 ? a[5] : a[6])));
        const float hi = o == -2 ? a[5] : (o == -1 ? a[4] : (o == 1 ? a[2] : (o == 2 ? a[1] : a[0])));
        return (up ? lo : hi) - f0;
    };
    const float e4 = s[4 * sg * st] - f0, e5 = s[5 * sg * st] - f0;
    if (code == 1 || code == -1) {
        const float e6 = s[6 * sg * st] - f0;
        return ((3.0f * w(-1) + 57.0f * w(1)) + (-90.0f * w(2) + 85.0f * w(3))) + ((-48.0f * e4 + 15.0f * e5) + -2.0f * e6);
    }
    return ((2.0f * w(-2) + -13.0f * w(-1)) + (-55.0f * w(1) + 50.0f * w(2))) + ((-27.0f * w(3) + 8.0f * e4) + -1.0f * e5);
}
// Shared-memory strides and this thread's centre in each box kind.
constexpr int V2X = AHZ * (AY + 4), V3X = AHZ * (AY + 6), SYB = AHZ;

// Where a box of kind `kind` starts relative to the tile origin (x0, y0, z0):
// halo 2 or 3 below the tile in x and y, 4 in z (a 16-byte origin).  A tile
// that holds the rows next to an upper Sommerfeld face starts its boxes
// lower, far enough for those rows' one-sided stencils (they reach 4 below
// the face in D1 and mixed D1, 5 in D2, 7 in the sixth difference); the box
// sizes still cover every valid sample's taps above.
__device__ __forceinline__ int upper_face_in(const Axis& A, int t0, int T, int blo, int bhi) {
    if (!A.rbc) return INT_MIN;
    const int xf = A.end - 1;
    const int lo = max(t0, max(xf - 2, blo)), hi = min(t0 + T - 1, min(xf - 1, bhi - 1));
    return lo <= hi ? xf : INT_MIN;
}
__device__ __forceinline__ void box_origin(int kind, int x0, int y0, int z0, const Geo& G, const Box& B, int& ox, int& oy,
                                           int& oz) {
    const int hx = (a_hx(kind) - AX) / 2, hy = (a_hy(kind) - AY) / 2;
    const int reach = kind == kBoxV3 ? 7 : (kind == kBoxV2 ? 5 : 4);   // below an upper face
    ox = -hx;
    oy = -hy;
    oz = -4;
    int f = hx ? upper_face_in(G.ax[0], x0, AX, B.lo[0], B.lo[0] + B.n[0]) : INT_MIN;
    if (f != INT_MIN) ox = min(ox, f - reach - x0);
    f = hy ? upper_face_in(G.ax[1], y0, AY, B.lo[1], B.lo[1] + B.n[1]) : INT_MIN;
    if (f != INT_MIN) oy = min(oy, f - reach - y0);
    f = upper_face_in(G.ax[2], z0, AZ, B.lo[2], B.lo[2] + B.n[2]);
    if (f != INT_MIN && f - reach - z0 < oz) oz = -((z0 - (f - reach) + 3) & ~3);
}
// Row code of index c along A (see d1_row): the upper face is checked first,
// as the forward's closures do.
__device__ __forceinline__ int row_code(const Axis& A, int c) {
    if (A.rbc) {
        const int r = A.end - 1 - c;
        if (r == 1 || r == 2) return -r;
    }
    if (A.lbc) {
        const int r = c - A.start;
        if (r == 1 || r == 2) return r;
    }
    return 0;
}

// The ring of one CTA: box ti is taken (its wait may give up: `missing`),
// read, and given back, after which its slot loads box ti + ANBUF.  give()
// is the CTA's one barrier per box; when any wait of the CTA gave up, the
// copies in flight get one more bounded wait and give() returns false, and
// the CTA leaves.  Stencils near Sommerfeld faces take the rows of this
// sample's row codes (codes, three fields of 3 bits).
template <int Seq>
struct BoxRing {
    const CurvMaps* maps;
    const Geo* G;
    const Box* B;
    float* ring;
    unsigned long long* bars;
    int* timeouts;
    int ntile, paired, nfield, z0, y0, x0, inst, t;
    int cV2, cDX, cDY, cV3;
    int codes;
    int ti;
    bool missing;

    __device__ __forceinline__ int code(int d) const { return ((codes >> (3 * d)) & 7) - 2; }
    __device__ __forceinline__ void issue(int i) {
        const CurvTile tl = seq_tile<Seq>(i, paired, nfield);
        const int b = i % ANBUF;
        int ox, oy, oz;
        box_origin(tl.kind, x0, y0, z0, *G, *B, ox, oy, oz);
        load_box(ring + b * (A_SLOT / 4), &maps->map[tl.kind], z0 + oz, y0 + oy, x0 + ox, inst, tl.comp, &bars[b],
                 a_bytes(tl.kind));
    }
    // A sample outside the box reads (and discards) as if it sat at the tile
    // origin with interior stencils: a box lowered for an upper face ends too
    // low for the tile's samples beyond that face.
    __device__ __forceinline__ void start(int tz, int ty, int tx, bool valid) {
        const int cx = valid ? x0 + tx : 0, cy = valid ? y0 + ty : 0, cz = valid ? z0 + tz : 0;
        if (!valid) tx = ty = tz = 0;
        auto centre = [&](int kind) {
            int ox, oy, oz;
            box_origin(kind, x0, y0, z0, *G, *B, ox, oy, oz);
            return ((tx - ox) * a_hy(kind) + (ty - oy)) * AHZ + (tz - oz);
        };
        cV2 = centre(kBoxV2);
        cDX = centre(kBoxDX);
        cDY = centre(kBoxDY);
        cV3 = centre(kBoxV3);
        codes = valid ? (row_code(G->ax[0], cx) + 2) | ((row_code(G->ax[1], cy) + 2) << 3)
                            | ((row_code(G->ax[2], cz) + 2) << 6)
                      : 2 | (2 << 3) | (2 << 6);
        ti = 0;
        missing = false;
        if (t == 0) {
            for (int b = 0; b < ANBUF; ++b) bar_init(&bars[b]);
            asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        }
        __syncthreads();
        if (t == 0)
            for (int i = 0; i < ANBUF && i < ntile; ++i) issue(i);
    }
    __device__ __forceinline__ const float* take() {
        const int b = ti % ANBUF;
        missing = missing || !bar_wait(&bars[b], (unsigned)((ti / ANBUF) & 1));
        return ring + b * (A_SLOT / 4);
    }
    __device__ __forceinline__ bool give() {
        if (__syncthreads_or(missing)) {
            if (t == 0) {
                atomicAdd(timeouts, 1);
                for (int i = ti; i < ti + ANBUF && i < ntile; ++i) bar_wait(&bars[i % ANBUF], (unsigned)((i / ANBUF) & 1));
            }
            return false;
        }
        if (t == 0 && ti + ANBUF < ntile) {
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            issue(ti + ANBUF);
        }
        ++ti;
        return true;
    }
    // The first derivative along axis d from the centre v of a box whose
    // stride along d is st.
    __device__ __forceinline__ float d1(const float* v, int st, int d) const {
        return d1_row(v, st, code(d), G->gf.d1a, G->gf.d1b, G->gf.inv_dx);
    }
    // The Hessian h[sym(i,j)] = d_i d_j f of the next Hessian group.
    __device__ __forceinline__ bool hessian(float (&h)[6]) {
        const float i12 = G->gf.inv_12dx2, idx2 = G->gf.inv_dx2;
        const float* v = take() + cV2;
        h[0] = d2_row(v, V2X, code(0), i12, idx2);
        h[3] = d2_row(v, SYB, code(1), i12, idx2);
        h[5] = d2_row(v, 1, code(2), i12, idx2);
        if (!give()) return false;
        if (paired) {
            v = take() + cV2;
            h[0] += d2_row(v, V2X, code(0), i12, idx2);
            h[3] += d2_row(v, SYB, code(1), i12, idx2);
            h[5] += d2_row(v, 1, code(2), i12, idx2);
            if (!give()) return false;
        }
        v = take() + cDX;
        h[1] = d1(v, SYB, 1);
        h[2] = d1(v, 1, 2);
        if (!give()) return false;
        v = take() + cDY;
        h[4] = d1(v, 1, 2);
        return give();
    }
    // Advection (upwind by the sign of beta; the centred or one-sided D1 on
    // the rows next to a Sommerfeld face) and the summed sixth-difference
    // numerators of the next halo-3 box, with its first derivatives when asked.
    __device__ __forceinline__ bool transport(const float (&beta)[3], float& adv, float& dis, float* d1out = nullptr) {
        const float inv12 = G->gf.inv_12dx, a1 = G->gf.d1a, a2 = G->gf.d1b;
        const float* v = take() + cV3;
        float ad[3], di[3];
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            const int st = d == 0 ? V3X : (d == 1 ? SYB : 1);
            const int c = code(d);
            float a[7];
#pragma unroll
            for (int o = 0; o < 7; ++o) a[o] = v[(o - 3) * st];
            if (c == 0) {
                ad[d] = beta[d] * inv12 * up1(a, beta[d]);
                di[d] = ko(a);
                if (d1out) d1out[d] = (a[4] - a[2]) * a1 + (a[5] - a[1]) * a2;
            } else {
                // the centred D1 on rows +-2, the one-sided one on rows +-1
                float g = (a[4] - a[2]) * a1 + (a[5] - a[1]) * a2;
                if (c == 1 || c == -1) {
                    const bool up = c > 0;
                    const float f0 = a[3];
                    const float b1 = up ? a[2] : a[4], f1 = up ? a[4] : a[2], f2 = up ? a[5] : a[1],
                                f3 = up ? a[6] : a[0];
                    const float u1 = ((-0.25f * (b1 - f0) + 1.5f * (f1 - f0)) + -0.5f * (f2 - f0))
                                     + (1.0f / 12.0f) * (f3 - f0);
                    g = (c > 0 ? u1 : -u1) * G->gf.inv_dx;
                }
                ad[d] = beta[d] * g;
                di[d] = ko_row(a, v, st, c);
                if (d1out) d1out[d] = g;
            }
        }
        adv = (ad[0] + ad[1]) + ad[2];
        dis = (di[0] + di[1]) + di[2];
        return give();
    }
};
}  // namespace tma

// dt At_ij = TF[S_ij + alpha W gt_ij (gt^mn d_m d_n W)] + Q_ij + adv + KO, with
//   S_ij = alpha W^2 (-1/2 gt^mn d_m d_n gt_ij + gt_k(i d_j) Gt^k)
//          + alpha W d_i d_j W - W^2 d_i d_j alpha,
// TF the trace-free part and Q the pointwise terms (Christoffel products, the
// first-derivative parts of the W and lapse Hessians, At algebra and Lie
// terms; JAX_BSSN/bssn/extrinsic_curvature.py:119-224, geometry.py:21-186).
__global__ void __launch_bounds__(tma::A_THREADS, 2)
k_rhs_at_tma(const __grid_constant__ tma::CurvMaps maps, const float* __restrict__ u, const double* __restrict__ u64,
             const float* __restrict__ d1, double* __restrict__ k, Geo G, Box B, int z_base, int tiles_z, int tiles_y,
             int nfield, int paired, int* __restrict__ timeouts) {
    using namespace tma;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    float* ring = reinterpret_cast<float*>(smem_raw);
    float* qbuf = ring + ANBUF * (A_SLOT / 4);   // [AT_NQ][A_THREADS]
    const int tile = blockIdx.x, inst = blockIdx.y;
    const int z0 = z_base + AZ * (tile % tiles_z);
    const int y0 = B.lo[1] + AY * ((tile / tiles_z) % tiles_y);
    const int x0 = B.lo[0] + AX * (tile / (tiles_z * tiles_y));
    const int t = threadIdx.x;
    const int tz = t & 31, ty = (t >> 5) & 3, tx = t >> 7;
    const int x = x0 + tx, y = y0 + ty, z = z0 + tz;
    const bool valid = x < B.lo[0] + B.n[0] && y < B.lo[1] + B.n[1] && z >= B.lo[2] && z < B.lo[2] + B.n[2];
    BoxRing<kSeqAt> R;
    R.maps = &maps;
    R.G = &G;
    R.B = &B;
    R.ring = ring;
    R.bars = reinterpret_cast<unsigned long long*>(qbuf + AT_NQ * A_THREADS);
    R.timeouts = timeouts;
    R.ntile = seq_tiles(kSeqAt, paired);
    R.paired = paired;
    R.nfield = nfield;
    R.z0 = z0;
    R.y0 = y0;
    R.x0 = x0;
    R.inst = inst;
    R.t = t;
    R.start(tz, ty, tx, valid);

    // ---- pointwise terms, while the first boxes load ----
    const long long cs = G.cs;
    const long long p = ((long long)x * G.ax[1].P + y) * G.ax[2].P + z + (long long)inst * G.istride;
    float g[6] = {1.0f, 0.0f, 0.0f, 1.0f, 0.0f, 1.0f}, gi[6] = {1.0f, 0.0f, 0.0f, 1.0f, 0.0f, 1.0f};
    float W = 1.0f, alpha = 1.0f;
    if (valid) {
#pragma unroll
        for (int s = 0; s < 6; ++s) g[s] = u[(GXX + s) * cs + p] + (unit_diagonal(s) ? 1.0f : 0.0f);
        inverse_metric(g, gi);
        W = static_cast<float>(u64[CW * cs + p]);
        alpha = static_cast<float>(u64[CALPHA * cs + p]);
        const float aW = alpha * W, W2 = W * W, aW2 = aW * W;
        // alpha K At_ij - 2 alpha At_ik gt^kl At_lj + Lie terms - 2/3 At_ij div
        // beta first, parked in shared memory (volatile, so that none of it
        // stays in registers across the Christoffel rows)
        volatile float* Q = qbuf + t;
        {
        const float K = static_cast<float>(u64[CK * cs + p]);
        float A[6];
#pragma unroll
        for (int s = 0; s < 6; ++s) A[s] = u[(AXX + s) * cs + p];
        float db[3][3];
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int j = 0; j < 3; ++j) db[i][j] = d1[((long long)(j * nfield + MIX_B + i)) * cs + p];
        const float div = db[0][0] + db[1][1] + db[2][2];
        float M[3][3];   // M[k][j] = gt^kl At_lj
#pragma unroll
        for (int kk = 0; kk < 3; ++kk)
#pragma unroll
            for (int j = 0; j < 3; ++j)
                M[kk][j] = gi[sym(kk, 0)] * A[sym(0, j)] + gi[sym(kk, 1)] * A[sym(1, j)] + gi[sym(kk, 2)] * A[sym(2, j)];
        const float aK = alpha * K, m2a = -2.0f * alpha, m23div = (-2.0f / 3.0f) * div;
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int j = i; j < 3; ++j) {
                float AgA = 0.0f, lie = 0.0f;
#pragma unroll
                for (int kk = 0; kk < 3; ++kk) {
                    AgA += A[sym(i, kk)] * M[kk][j];
                    lie += A[sym(kk, i)] * db[kk][j] + A[sym(kk, j)] * db[kk][i];
                }
                const int s = sym(i, j);
                Q[s * A_THREADS] = (aK * A[s] + m2a * AgA) + lie + m23div * A[s];
            }
        }
        float PT[6];   // pointwise part of [alpha W^2 R_ij - W^2 D_i D_j alpha]
        {
            float c1[3][6];
            {
                float dg[3][6];
#pragma unroll
                for (int kk = 0; kk < 3; ++kk)
#pragma unroll
                    for (int s = 0; s < 6; ++s) dg[kk][s] = d1[((long long)(kk * nfield + MIX_G + s)) * cs + p];
                christoffel_first(dg, c1);
            }
            float dW[3], da[3];
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                dW[d] = d1[((long long)(d * nfield + MIX_W)) * cs + p];
                da[d] = d1[((long long)(d * nfield + MIX_ALPHA)) * cs + p];
            }
            {   // 1/2 Gt^m d_m gt_ij = 1/2 Gt^m (Gamma_ijm + Gamma_jim)
                const float Gt[3] = {u[GTX * cs + p], u[GTY * cs + p], u[GTZ * cs + p]};
                const float h = 0.5f * aW2;
#pragma unroll
                for (int i = 0; i < 3; ++i)
#pragma unroll
                    for (int j = i; j < 3; ++j) {
                        float t3 = 0.0f;
#pragma unroll
                        for (int m = 0; m < 3; ++m) t3 += Gt[m] * (c1[i][sym(j, m)] + c1[j][sym(i, m)]);
                        PT[sym(i, j)] = h * t3;
                    }
            }
            // One row Gamma^k_ij of the second kind at a time: the Christoffel
            // products (term4 + term5 of the conformal Ricci tensor) and the
            // first-derivative parts Gamma^k_ij d_k W, Gamma^k_ij d_k alpha of
            // the W and lapse Hessians.
            float gicW = 0.0f;   // gt^ij Gamma^k_ij d_k W
#pragma unroll
            for (int kk = 0; kk < 3; ++kk) {
                float c2k[6];
#pragma unroll
                for (int s = 0; s < 6; ++s)
                    c2k[s] = gi[sym(kk, 0)] * c1[0][s] + gi[sym(kk, 1)] * c1[1][s] + gi[sym(kk, 2)] * c1[2][s];
                gicW += dW[kk] * contract_sym(gi, c2k);
                const float ck = W2 * da[kk] - aW * dW[kk];
                // X[n][b] = gt^na Gamma^k_ab, one column b at a time (three
                // columns live instead of nine).
                auto xcol = [&](int b, float (&xc)[3]) {
#pragma unroll
                    for (int n = 0; n < 3; ++n)
                        xc[n] = gi[sym(0, n)] * c2k[sym(0, b)] + gi[sym(1, n)] * c2k[sym(1, b)]
                                + gi[sym(2, n)] * c2k[sym(2, b)];
                };
#pragma unroll
                for (int i = 0; i < 3; ++i) {
                    float xi[3];
                    xcol(i, xi);
#pragma unroll
                    for (int j = i; j < 3; ++j) {
                        float xj[3];
                        if (j == i) {
#pragma unroll
                            for (int n = 0; n < 3; ++n) xj[n] = xi[n];
                        } else {
                            xcol(j, xj);
                        }
                        float acc = 0.0f;
#pragma unroll
                        for (int n = 0; n < 3; ++n)
                            acc += xi[n] * (c1[j][sym(kk, n)] + c1[kk][sym(j, n)]) + xj[n] * c1[i][sym(kk, n)];
                        const int s = sym(i, j);
                        PT[s] += aW2 * acc + c2k[s] * ck;
                    }
                }
            }
            // gt_ij is read again (an L1 hit) rather than held across the
            // Christoffel rows
#pragma unroll
            for (int s = 0; s < 6; ++s) g[s] = reload(u + (GXX + s) * cs + p) + (unit_diagonal(s) ? 1.0f : 0.0f);
            float grad2 = 0.0f, gw = 0.0f;   // gt^mn d_m W d_n W, gt^mn d_m W d_n alpha
#pragma unroll
            for (int n = 0; n < 3; ++n) {
                const float gdw = gi[sym(0, n)] * dW[0] + gi[sym(1, n)] * dW[1] + gi[sym(2, n)] * dW[2];
                grad2 += gdw * dW[n];
                gw += gdw * da[n];
            }
#pragma unroll
            for (int i = 0; i < 3; ++i)
#pragma unroll
                for (int j = i; j < 3; ++j) {
                    const int s = sym(i, j);
                    const float grad = dW[i] * da[j] + dW[j] * da[i] - g[s] * gw;
                    PT[s] += -g[s] * (aW * gicW + 2.0f * alpha * grad2) - W * grad;
                }
        }
        const float trP = contract_sym(gi, PT);
#pragma unroll
        for (int s = 0; s < 6; ++s) Q[s * A_THREADS] += PT[s] - (1.0f / 3.0f) * g[s] * trP;
    } else {
#pragma unroll
        for (int s = 0; s < AT_NQ; ++s) qbuf[s * A_THREADS + t] = 0.0f;
    }

    // ---- the boxes ----
    const float aW = alpha * W, W2 = W * W, aW2 = aW * W;
    float S[6] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
    float L = 0.0f;   // gt^mn d_m d_n W (stencil parts)
    // Hessians of gt_ij (-1/2 alpha W^2 gt^mn d_m d_n gt_ij), W (alpha W d_i d_j W
    // and its trace) and alpha (-W^2 d_i d_j alpha)
#pragma unroll 1
    for (int f = 0; f < 8; ++f) {
        float h[6];
        if (!R.hessian(h)) return;
        if (f < 6) {
            const float r = -aW2 * (0.5f * ((gi[0] * h[0] + gi[3] * h[3]) + gi[5] * h[5])
                                    + ((gi[1] * h[1] + gi[2] * h[2]) + gi[4] * h[4]));
#pragma unroll
            for (int q = 0; q < 6; ++q)
                if (q == f) S[q] += r;
        } else {
            if (f == 6) L = contract_sym(gi, h);
            const float c = f == 6 ? aW : -W2;
#pragma unroll
            for (int q = 0; q < 6; ++q) S[q] += c * h[q];
        }
    }
#pragma unroll
    for (int m = 0; m < 3; ++m) {   // alpha W^2 gt_k(i d_j) Gt^k
        const float* v = R.take() + R.cV2;
        const float e[3] = {0.5f * aW2 * R.d1(v, V2X, 0), 0.5f * aW2 * R.d1(v, SYB, 1), 0.5f * aW2 * R.d1(v, 1, 2)};
        if (!R.give()) return;
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int j = i; j < 3; ++j) S[sym(i, j)] += g[sym(m, i)] * e[j] + g[sym(m, j)] * e[i];
    }
    {   // the trace-free part plus the pointwise terms, back into qbuf
#pragma unroll
        for (int s = 0; s < 6; ++s) S[s] += aW * g[s] * L;
        const float tr = contract_sym(gi, S);
#pragma unroll
        for (int s = 0; s < 6; ++s) qbuf[s * A_THREADS + t] += S[s] - (1.0f / 3.0f) * g[s] * tr;
    }
    float beta[3] = {0.0f, 0.0f, 0.0f};
    if (valid)
#pragma unroll
        for (int d = 0; d < 3; ++d) beta[d] = static_cast<float>(u64[(BX + d) * cs + p]);
    const float scale = G.gf.ko_scale;
#pragma unroll 1
    for (int s = 0; s < 6; ++s) {   // advection and dissipation of At_ij
        float adv, dis;
        if (!R.transport(beta, adv, dis)) return;
        if (valid) k[(AXX + s) * cs + p] = (qbuf[s * A_THREADS + t] + adv) + scale * dis;
    }
}

// dt K    = -W^2 gt^mn d_m d_n alpha + PK + adv + KO,
// dt Gt^i = gt^mn d_m d_n beta^i + 1/3 gt^ij d_j d_l beta^l - 4/3 alpha gt^ij d_j K
//           + PG^i + adv + KO,
// PK and PG^i the pointwise terms (JAX_BSSN/bssn/extrinsic_curvature.py:31-92,
// conformal_connection.py:19-162).
__global__ void __launch_bounds__(tma::A_THREADS, 2)
k_rhs_kgt_tma(const __grid_constant__ tma::CurvMaps maps, const float* __restrict__ u, const double* __restrict__ u64,
              const float* __restrict__ d1, double* __restrict__ k, Geo G, Box B, int z_base, int tiles_z,
              int tiles_y, int nfield, int paired, int* __restrict__ timeouts) {
    using namespace tma;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    float* ring = reinterpret_cast<float*>(smem_raw);
    float* qbuf = ring + ANBUF * (A_SLOT / 4);   // [KGT_NQ][A_THREADS]: PK, PG^0..2
    const int tile = blockIdx.x, inst = blockIdx.y;
    const int z0 = z_base + AZ * (tile % tiles_z);
    const int y0 = B.lo[1] + AY * ((tile / tiles_z) % tiles_y);
    const int x0 = B.lo[0] + AX * (tile / (tiles_z * tiles_y));
    const int t = threadIdx.x;
    const int tz = t & 31, ty = (t >> 5) & 3, tx = t >> 7;
    const int x = x0 + tx, y = y0 + ty, z = z0 + tz;
    const bool valid = x < B.lo[0] + B.n[0] && y < B.lo[1] + B.n[1] && z >= B.lo[2] && z < B.lo[2] + B.n[2];
    BoxRing<kSeqKgt> R;
    R.maps = &maps;
    R.G = &G;
    R.B = &B;
    R.ring = ring;
    R.bars = reinterpret_cast<unsigned long long*>(qbuf + KGT_NQ * A_THREADS);
    R.timeouts = timeouts;
    R.ntile = seq_tiles(kSeqKgt, paired);
    R.paired = paired;
    R.nfield = nfield;
    R.z0 = z0;
    R.y0 = y0;
    R.x0 = x0;
    R.inst = inst;
    R.t = t;
    R.start(tz, ty, tx, valid);

    // ---- pointwise terms, while the first boxes load ----
    const long long cs = G.cs;
    const long long p = ((long long)x * G.ax[1].P + y) * G.ax[2].P + z + (long long)inst * G.istride;
    float gi[6] = {1.0f, 0.0f, 0.0f, 1.0f, 0.0f, 1.0f};
    float W = 1.0f, alpha = 1.0f;
    if (valid) {
        float g[6];
#pragma unroll
        for (int s = 0; s < 6; ++s) g[s] = u[(GXX + s) * cs + p] + (unit_diagonal(s) ? 1.0f : 0.0f);
        inverse_metric(g, gi);
        W = static_cast<float>(u64[CW * cs + p]);
        alpha = static_cast<float>(u64[CALPHA * cs + p]);
        const float K = static_cast<float>(u64[CK * cs + p]);
        float c1[3][6];
        {
            float dg[3][6];
#pragma unroll
            for (int kk = 0; kk < 3; ++kk)
#pragma unroll
                for (int s = 0; s < 6; ++s) dg[kk][s] = d1[((long long)(kk * nfield + MIX_G + s)) * cs + p];
            christoffel_first(dg, c1);
        }
        float dW[3], da[3];
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            dW[d] = d1[((long long)(d * nfield + MIX_W)) * cs + p];
            da[d] = d1[((long long)(d * nfield + MIX_ALPHA)) * cs + p];
        }
        float A[6], Au[6];   // Au = A^ij = gt^ik (A_kl gt^lj)
#pragma unroll
        for (int s = 0; s < 6; ++s) A[s] = u[(AXX + s) * cs + p];
        {
            float M[3][3];
#pragma unroll
            for (int kk = 0; kk < 3; ++kk)
#pragma unroll
                for (int j = 0; j < 3; ++j)
                    M[kk][j] = A[sym(kk, 0)] * gi[sym(0, j)] + A[sym(kk, 1)] * gi[sym(1, j)] + A[sym(kk, 2)] * gi[sym(2, j)];
#pragma unroll
            for (int i = 0; i < 3; ++i)
#pragma unroll
                for (int j = i; j < 3; ++j)
                    Au[sym(i, j)] = gi[sym(i, 0)] * M[0][j] + gi[sym(i, 1)] * M[1][j] + gi[sym(i, 2)] * M[2][j];
        }
        // One row Gamma^i_jk of the second kind at a time: Gamma^i_jk A^jk (dt Gt^i)
        // and gt^jk Gamma^i_jk d_i alpha (dt K)
        float t2[3], gicA = 0.0f;
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            float c2i[6];
#pragma unroll
            for (int s = 0; s < 6; ++s)
                c2i[s] = gi[sym(i, 0)] * c1[0][s] + gi[sym(i, 1)] * c1[1][s] + gi[sym(i, 2)] * c1[2][s];
            t2[i] = contract_sym(c2i, Au);
            gicA += da[i] * contract_sym(gi, c2i);
        }
        {   // dt K: gt^ij (W^2 Gamma^m_ij d_m alpha - W grad_ij) + alpha At_ij A^ij + alpha K^2 / 3
            float gw = 0.0f;
#pragma unroll
            for (int n = 0; n < 3; ++n) gw += (gi[sym(0, n)] * dW[0] + gi[sym(1, n)] * dW[1] + gi[sym(2, n)] * dW[2]) * da[n];
            float gr[6];
#pragma unroll
            for (int i = 0; i < 3; ++i)
#pragma unroll
                for (int j = i; j < 3; ++j) gr[sym(i, j)] = dW[i] * da[j] + dW[j] * da[i] - g[sym(i, j)] * gw;
            qbuf[t] = ((W * W) * gicA - W * contract_sym(gi, gr)) + alpha * contract_sym(A, Au) + alpha * (K * K) / 3.0f;
        }
        {   // dt Gt^i: 2 alpha Gamma^i_jk A^jk - 6 alpha/W A^ij d_j W - 2 A^ij d_j alpha
            //          + 2/3 Gt^i div beta - Gt^j d_j beta^i
            float db[3][3];
#pragma unroll
            for (int i = 0; i < 3; ++i)
#pragma unroll
                for (int j = 0; j < 3; ++j) db[i][j] = d1[((long long)(j * nfield + MIX_B + i)) * cs + p];
            const float div = db[0][0] + db[1][1] + db[2][2];
            const float six_alpha_over_w = -6.0f * alpha * static_cast<float>(1.0 / fmax(u64[CW * cs + p], 1.0e-12));
            const float Gt[3] = {u[GTX * cs + p], u[GTY * cs + p], u[GTZ * cs + p]};
#pragma unroll
            for (int i = 0; i < 3; ++i) {
                float t3 = 0.0f, t4 = 0.0f, t7 = 0.0f;
#pragma unroll
                for (int j = 0; j < 3; ++j) {
                    t3 += Au[sym(i, j)] * dW[j];
                    t4 += Au[sym(i, j)] * da[j];
                    t7 += Gt[j] * db[i][j];
                }
                qbuf[(1 + i) * A_THREADS + t] = (((2.0f * alpha) * t2[i] + six_alpha_over_w * t3) - 2.0f * t4)
                                                + ((2.0f / 3.0f) * Gt[i] * div - t7);
            }
        }
    } else {
#pragma unroll
        for (int q = 0; q < KGT_NQ; ++q) qbuf[q * A_THREADS + t] = 0.0f;
    }

    // ---- the boxes ----
    float accK = 0.0f;
    float accG[3] = {0.0f, 0.0f, 0.0f};
    float graddiv[3] = {0.0f, 0.0f, 0.0f};   // d_m d_l beta^l
    // Hessians of alpha (-W^2 gt^mn d_m d_n alpha) and beta^l (gt^mn d_m d_n beta^l)
#pragma unroll 1
    for (int f = 0; f < 4; ++f) {
        float h[6];
        if (!R.hessian(h)) return;
        const float c = contract_sym(gi, h);
        if (f == 0) {
            accK = -(W * W) * c;
        } else {
#pragma unroll
            for (int l = 0; l < 3; ++l)
                if (l == f - 1) {
                    accG[l] += c;
#pragma unroll
                    for (int m = 0; m < 3; ++m) graddiv[m] += h[sym(m, l)];
                }
        }
    }
    float beta[3] = {0.0f, 0.0f, 0.0f};
    if (valid)
#pragma unroll
        for (int d = 0; d < 3; ++d) beta[d] = static_cast<float>(u64[(BX + d) * cs + p]);
    const float scale = G.gf.ko_scale;
    {   // K: its first derivatives, advection and dissipation
        float adv, dis, dK[3];
        if (!R.transport(beta, adv, dis, dK)) return;
        if (valid) k[CK * cs + p] = ((accK + qbuf[t]) + adv) + scale * dis;
        const float m43a = (-4.0f / 3.0f) * alpha;
#pragma unroll
        for (int i = 0; i < 3; ++i)
            accG[i] += m43a * (gi[sym(i, 0)] * dK[0] + gi[sym(i, 1)] * dK[1] + gi[sym(i, 2)] * dK[2])
                       + (1.0f / 3.0f) * (gi[sym(i, 0)] * graddiv[0] + gi[sym(i, 1)] * graddiv[1]
                                          + gi[sym(i, 2)] * graddiv[2]);
    }
#pragma unroll
    for (int i = 0; i < 3; ++i) {   // Gt^i: advection and dissipation
        float adv, dis;
        if (!R.transport(beta, adv, dis)) return;
        if (valid) k[(GTX + i) * cs + p] = ((accG[i] + qbuf[(1 + i) * A_THREADS + t]) + adv) + scale * dis;
    }
}

// dt gt_ij, dt W, dt alpha, dt beta^i (JAX_BSSN/bssn/spatial_metric.py:17-106,
// shift_and_lapse.py:65-132): each field's pointwise part (Lie terms,
// slicing, Gamma-driver) in registers, then its advection and dissipation
// from its halo-3 box.  Same terms as k_rhs_gauge<float, false>.
__global__ void __launch_bounds__(tma::A_THREADS, 2)
k_rhs_gauge_tma(const __grid_constant__ tma::CurvMaps maps, const float* __restrict__ u, const double* __restrict__ u64,
                const float* __restrict__ d1, double* __restrict__ k, Geo G, Box B, int z_base, int tiles_z,
                int tiles_y, int nfield, int paired, int* __restrict__ timeouts) {
    using namespace tma;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    float* ring = reinterpret_cast<float*>(smem_raw);
    const int tile = blockIdx.x, inst = blockIdx.y;
    const int z0 = z_base + AZ * (tile % tiles_z);
    const int y0 = B.lo[1] + AY * ((tile / tiles_z) % tiles_y);
    const int x0 = B.lo[0] + AX * (tile / (tiles_z * tiles_y));
    const int t = threadIdx.x;
    const int tz = t & 31, ty = (t >> 5) & 3, tx = t >> 7;
    const int x = x0 + tx, y = y0 + ty, z = z0 + tz;
    const bool valid = x < B.lo[0] + B.n[0] && y < B.lo[1] + B.n[1] && z >= B.lo[2] && z < B.lo[2] + B.n[2];
    BoxRing<kSeqGauge> R;
    R.maps = &maps;
    R.G = &G;
    R.B = &B;
    R.ring = ring;
    R.bars = reinterpret_cast<unsigned long long*>(ring + ANBUF * (A_SLOT / 4));
    R.timeouts = timeouts;
    R.ntile = seq_tiles(kSeqGauge, paired);
    R.paired = paired;
    R.nfield = nfield;
    R.z0 = z0;
    R.y0 = y0;
    R.x0 = x0;
    R.inst = inst;
    R.t = t;
    R.start(tz, ty, tx, valid);

    const long long cs = G.cs;
    const long long p = ((long long)x * G.ax[1].P + y) * G.ax[2].P + z + (long long)inst * G.istride;
    float P[NMIX], beta[3] = {0.0f, 0.0f, 0.0f};
#pragma unroll
    for (int f = 0; f < NMIX; ++f) P[f] = 0.0f;
    if (valid) {
#pragma unroll
        for (int d = 0; d < 3; ++d) beta[d] = static_cast<float>(u64[(BX + d) * cs + p]);
        float db[3][3];   // db[i][j] = d_j beta^i
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int j = 0; j < 3; ++j) db[i][j] = d1[((long long)(j * nfield + MIX_B + i)) * cs + p];
        const float div = db[0][0] + db[1][1] + db[2][2];
        const float alpha = static_cast<float>(u64[CALPHA * cs + p]);
        const float K = static_cast<float>(u64[CK * cs + p]);
        const float W = static_cast<float>(u64[CW * cs + p]);
        float g[6];
#pragma unroll
        for (int s = 0; s < 6; ++s) g[s] = u[(GXX + s) * cs + p] + (unit_diagonal(s) ? 1.0f : 0.0f);
        const float m23div = (-2.0f / 3.0f) * div, m2a = -2.0f * alpha;
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int j = i; j < 3; ++j) {
                float lie = 0.0f;
#pragma unroll
                for (int m = 0; m < 3; ++m) lie += g[sym(m, i)] * db[m][j] + g[sym(m, j)] * db[m][i];
                const int s = sym(i, j);
                P[s] = lie + m23div * g[s] + m2a * u[(AXX + s) * cs + p];
            }
        P[MIX_W] = (1.0f / 3.0f) * alpha * W * K - (1.0f / 3.0f) * W * div;
        P[MIX_ALPHA] = (G.gauge == 0) ? -(alpha * alpha) * K : -2.0f * alpha * K;
#pragma unroll
        for (int i = 0; i < 3; ++i)
            P[MIX_B + i] = G.zero_shift ? 0.0f * beta[i] : G.gf.g * u[(GTX + i) * cs + p] + (-G.gf.eta) * beta[i];
    }
    const float scale = G.gf.ko_scale;
#pragma unroll 1
    for (int f = 0; f < NMIX; ++f) {
        float adv, dis;
        if (!R.transport(beta, adv, dis)) return;
        float pf = P[0];
#pragma unroll
        for (int q = 1; q < NMIX; ++q) pf = q == f ? P[q] : pf;
        float v;
        if (f >= MIX_B && G.zero_shift) v = pf;
        else if (f == MIX_ALPHA) v = (pf + adv) + scale * dis;
        else v = (adv + pf) + scale * dis;
        if (valid && !R.missing) k[mix_source(f) * cs + p] = v;
    }
}

// ---------------------------------------------------------------------------
// dt K and dt Gt^i
// ---------------------------------------------------------------------------
template <typename R, bool Closed>
__global__ void __launch_bounds__(kThreads, kMinBlocks<R>)
k_rhs_kgt(const R* __restrict__ u, const double* __restrict__ u64, const R* __restrict__ d1,
          const double* __restrict__ mat, double* __restrict__ k, Geo G, BoxSet S, int nfield) {
    PointCtx c;
    if (!point<Closed>(S.b[blockIdx.y], c, G)) return;
    const long long cs = G.cs, p = c.p;
    R g[6], gi[6];
    load_sym(u, GXX, G, c, g);
    inverse_metric(g, gi);
    R c1[3][6], c2[3][6];
    {
        R dg[3][6];
        load_metric_derivs(d1, G, nfield, p, dg);
        christoffel(dg, gi, c1, c2);
    }
    R dW[3], da[3], dK[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        dW[d] = d1ptr(d1, G, nfield, d, MIX_W, p)[0];
        da[d] = d1ptr(d1, G, nfield, d, MIX_ALPHA, p)[0];
        dK[d] = D1<R, Closed>(u + CK * cs + p, G, d, c.ix[d]);
    }
    const R W = full_exact(u, u64, CW, cs, p);
    const R alpha = full_exact(u, u64, CALPHA, cs, p);
    const R K = full_exact(u, u64, CK, cs, p);
    const R beta[3] = {full_exact(u, u64, BX, cs, p), full_exact(u, u64, BY, cs, p), full_exact(u, u64, BZ, cs, p)};
    R bs[3];
    shift_over_12dx(G, beta, bs);
    R A[6];
    load_sym(u, AXX, G, c, A);
    R Au[6];  // A^ij = g^ik (A_kl g^lj)
    {
        R M[3][3];  // M[k][j] = A_kl g^lj
#pragma unroll
        for (int kk = 0; kk < 3; ++kk)
#pragma unroll
            for (int j = 0; j < 3; ++j)
                M[kk][j] = A[sym(kk, 0)] * gi[sym(0, j)] + A[sym(kk, 1)] * gi[sym(1, j)] + A[sym(kk, 2)] * gi[sym(2, j)];
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int j = i; j < 3; ++j)
                Au[sym(i, j)] = gi[sym(i, 0)] * M[0][j] + gi[sym(i, 1)] * M[1][j] + gi[sym(i, 2)] * M[2][j];
    }

    // dt K
    {
        R h[6];
        w2_lapse_hessian<R, Closed>(u, d1, G, nfield, c, g, gi, c2, dW, da, W, h);
        const R first = -contract_sym(gi, h);
        const R second = alpha * contract_sym(A, Au);
        const R third = alpha * (K * K) / R(3.0);
        const R* f = u + CK * cs + p;
        R bulk = first + second + third + ADV<R, Closed, false>(f, G, c.ix, beta, bs);
        if (mat != nullptr) {
            // + 4 pi alpha (rho + W^2 gt^ij S_ij) (extrinsic_curvature.py:78-87)
            const R wf = static_cast<R>(fmax(u64[CW * cs + p], 1.0e-12));
            const R wf2 = wf * wf;
            R trace = R(0);
#pragma unroll
            for (int i = 0; i < 3; ++i)
#pragma unroll
                for (int j = 0; j < 3; ++j) trace += (wf2 * gi[sym(i, j)]) * static_cast<R>(mat[(4 + sym(i, j)) * cs + p]);
            bulk = bulk + R(4.0 * kPi) * alpha * (static_cast<R>(mat[p]) + trace);
        }
        k[CK * cs + p] = bulk + KO<R, Closed, false>(f, G, c.ix);
    }

    // dt Gt^i
    R db[3][3];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) db[i][j] = d1ptr(d1, G, nfield, j, MIX_B + i, p)[0];
    const R div = db[0][0] + db[1][1] + db[2][2];
    // -6 alpha / max(W, 1e-12); the FP32 form takes 1/W in FP64 (puncture values)
    R six_alpha_over_w;
    if constexpr (kPerturbative<R>) {
        six_alpha_over_w = R(-6.0) * alpha * static_cast<R>(1.0 / fmax(u64[CW * cs + p], 1.0e-12));
    } else {
        const R Wf = fmax(W, 1.0e-12);
        six_alpha_over_w = -6.0 * alpha / Wf;
    }
    R hb[3][6];  // hb[i][sym(m,n)] = d_m d_n beta^i
#pragma unroll 1
    for (int i = 0; i < 3; ++i) hessian<R, Closed, kExactBg<R>>(u, d1, G, nfield, BX + i, MIX_B + i, c, hb[i]);
    R graddiv[3];
#pragma unroll
    for (int m = 0; m < 3; ++m) graddiv[m] = hb[0][sym(m, 0)] + hb[1][sym(m, 1)] + hb[2][sym(m, 2)];
    const R Gt[3] = {full(u, GTX, G, c), full(u, GTY, G, c), full(u, GTZ, G, c)};
#pragma unroll 1
    for (int i = 0; i < 3; ++i) {
        R t1 = R(0), t3 = R(0), t4 = R(0), t7 = R(0), t9 = R(0);
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            t1 += gi[sym(i, j)] * dK[j];
            t3 += Au[sym(i, j)] * dW[j];
            t4 += Au[sym(i, j)] * da[j];
            t7 += Gt[j] * db[i][j];
            t9 += gi[sym(i, j)] * graddiv[j];
        }
        const R t2 = contract_sym(c2[i], Au);
        const R t8 = contract_sym(gi, hb[i]);
        const R* f = u + (GTX + i) * cs + p;
        const R v = R(-4.0 / 3.0) * alpha * t1 + R(2.0) * alpha * t2 + six_alpha_over_w * t3
                    - R(2.0) * t4 + ADV<R, Closed, false>(f, G, c.ix, beta, bs) + R(2.0 / 3.0) * Gt[i] * div - t7 + t8
                    + R(1.0 / 3.0) * t9;
        R out = v + KO<R, Closed, false>(f, G, c.ix);
        if (mat != nullptr) {
            // - 16 pi alpha gt^ij S_j (conformal_connection.py:166-178)
            R gs = R(0);
#pragma unroll
            for (int j = 0; j < 3; ++j) gs += gi[sym(i, j)] * static_cast<R>(mat[(1 + j) * cs + p]);
            out = out + R(-16.0 * kPi) * alpha * gs;
        }
        k[(GTX + i) * cs + p] = out;
    }
}

// ---------------------------------------------------------------------------
// dt At_ij
// ---------------------------------------------------------------------------
template <typename R, bool Closed>
__global__ void __launch_bounds__(kThreads, kMinBlocks<R>)
k_rhs_at(const R* __restrict__ u, const double* __restrict__ u64, const R* __restrict__ d1,
         const R* __restrict__ damp, const double* __restrict__ mat, double* __restrict__ k, Geo G, BoxSet S,
         int nfield) {
    PointCtx c;
    if (!point<Closed>(S.b[blockIdx.y], c, G)) return;
    const long long cs = G.cs, p = c.p;
    R g[6], gi[6];
    load_sym(u, GXX, G, c, g);
    inverse_metric(g, gi);
    R c1[3][6], c2[3][6];
    {
        R dg[3][6];
        load_metric_derivs(d1, G, nfield, p, dg);
        christoffel(dg, gi, c1, c2);
    }
    R dW[3], da[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        dW[d] = d1ptr(d1, G, nfield, d, MIX_W, p)[0];
        da[d] = d1ptr(d1, G, nfield, d, MIX_ALPHA, p)[0];
    }
    const R W = full_exact(u, u64, CW, cs, p);
    const R alpha = full_exact(u, u64, CALPHA, cs, p);

    R w2r[6];
    w2_ricci<R, Closed>(u, d1, G, nfield, c, g, gi, c1, c2, dW, W, w2r);
    // --- [alpha W^2 R_ij - W^2 D_i D_j alpha]^TF ---
    R T[6];
    {
        R h[6];
        w2_lapse_hessian<R, Closed>(u, d1, G, nfield, c, g, gi, c2, dW, da, W, h);
#pragma unroll
        for (int s = 0; s < 6; ++s) T[s] = alpha * w2r[s] - h[s];
        if (mat != nullptr) {
            // - 8 pi alpha W^2 S_ij before the trace-free part (extrinsic_curvature.py:164-175)
            const R wf = static_cast<R>(fmax(u64[CW * cs + p], 1.0e-12));
            const R coef = R(8.0 * kPi) * alpha * (wf * wf);
#pragma unroll
            for (int s = 0; s < 6; ++s) T[s] = T[s] - coef * static_cast<R>(mat[(4 + s) * cs + p]);
        }
        const R tr = contract_sym(gi, T);
#pragma unroll
        for (int s = 0; s < 6; ++s) T[s] = T[s] - R(1.0 / 3.0) * g[s] * tr;
    }
    // --- remaining terms ---
    const R K = full_exact(u, u64, CK, cs, p);
    R A[6];
    load_sym(u, AXX, G, c, A);
    const R beta[3] = {full_exact(u, u64, BX, cs, p), full_exact(u, u64, BY, cs, p), full_exact(u, u64, BZ, cs, p)};
    R bs[3];
    shift_over_12dx(G, beta, bs);
    R db[3][3];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) db[i][j] = d1ptr(d1, G, nfield, j, MIX_B + i, p)[0];
    const R div = db[0][0] + db[1][1] + db[2][2];
    {
        // Pointwise terms of every component first, with static indices:
        // alpha K A_ij - 2 alpha A_ik g^kl A_lj + Lie terms - 2/3 A_ij div beta.
        R M[3][3];  // M[k][j] = g^kl A_lj
#pragma unroll
        for (int kk = 0; kk < 3; ++kk)
#pragma unroll
            for (int j = 0; j < 3; ++j)
                M[kk][j] = gi[sym(kk, 0)] * A[sym(0, j)] + gi[sym(kk, 1)] * A[sym(1, j)] + gi[sym(kk, 2)] * A[sym(2, j)];
        const R aK = alpha * K, m2a = R(-2.0) * alpha, m23div = R(-2.0 / 3.0) * div;
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int j = i; j < 3; ++j) {
                R AgA = R(0), lie = R(0);
#pragma unroll
                for (int kk = 0; kk < 3; ++kk) {
                    AgA += A[sym(i, kk)] * M[kk][j];
                    lie += A[sym(kk, i)] * db[kk][j] + A[sym(kk, j)] * db[kk][i];
                }
                const int s = sym(i, j);
                T[s] = (aK * A[s] + m2a * AgA) + T[s] + lie + m23div * A[s];
            }
    }
#pragma unroll 1
    for (int s = 0; s < 6; ++s) {
        const R* f = u + (AXX + s) * cs + p;
        R v = T[s] + ADV<R, Closed, false>(f, G, c.ix, beta, bs);
        if (damp != nullptr) v += damp[s * cs + p];
        k[(AXX + s) * cs + p] = v + KO<R, Closed, false>(f, G, c.ix);
    }
}

// ---------------------------------------------------------------------------
// dt K, dt Gt^i and dt At_ij in one pass (the FP64 form).  The two curvature
// kernels above share the inverse metric, the Christoffel symbols, the lapse
// Hessian and the products of At with gt^ij; the FP64 form is bound by its
// FP64 instruction count, not by occupancy, so it computes those once.
// ---------------------------------------------------------------------------
template <typename R, bool Closed>
__global__ void __launch_bounds__(kThreads)
k_rhs_curv(const R* __restrict__ u, const double* __restrict__ u64, const R* __restrict__ d1,
           const R* __restrict__ damp, const double* __restrict__ mat, double* __restrict__ k, Geo G, BoxSet S,
           int nfield) {
    PointCtx c;
    if (!point<Closed>(S.b[blockIdx.y], c, G)) return;
    const long long cs = G.cs, p = c.p;
    R g[6], gi[6];
    load_sym(u, GXX, G, c, g);
    inverse_metric(g, gi);
    R c1[3][6], c2[3][6];
    {
        R dg[3][6];
        load_metric_derivs(d1, G, nfield, p, dg);
        christoffel(dg, gi, c1, c2);
    }
    R dW[3], da[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        dW[d] = d1ptr(d1, G, nfield, d, MIX_W, p)[0];
        da[d] = d1ptr(d1, G, nfield, d, MIX_ALPHA, p)[0];
    }
    const R W = full_exact(u, u64, CW, cs, p);
    const R alpha = full_exact(u, u64, CALPHA, cs, p);

    // [alpha W^2 R_ij - W^2 D_i D_j alpha]^TF and gt^ij W^2 D_i D_j alpha
    R T[6], lapse_lap;
    {
        R w2r[6];
        w2_ricci<R, Closed>(u, d1, G, nfield, c, g, gi, c1, c2, dW, W, w2r);
        R h[6];
        w2_lapse_hessian<R, Closed>(u, d1, G, nfield, c, g, gi, c2, dW, da, W, h);
        lapse_lap = contract_sym(gi, h);
#pragma unroll
        for (int s = 0; s < 6; ++s) T[s] = alpha * w2r[s] - h[s];
        if (mat != nullptr) {
            const R wf = static_cast<R>(fmax(u64[CW * cs + p], 1.0e-12));
            const R coef = R(8.0 * kPi) * alpha * (wf * wf);
#pragma unroll
            for (int s = 0; s < 6; ++s) T[s] = T[s] - coef * static_cast<R>(mat[(4 + s) * cs + p]);
        }
        const R tr = contract_sym(gi, T);
#pragma unroll
        for (int s = 0; s < 6; ++s) T[s] = T[s] - R(1.0 / 3.0) * g[s] * tr;
    }
    const R K = full_exact(u, u64, CK, cs, p);
    R A[6];
    load_sym(u, AXX, G, c, A);
    const R beta[3] = {full_exact(u, u64, BX, cs, p), full_exact(u, u64, BY, cs, p), full_exact(u, u64, BZ, cs, p)};
    R bs[3];
    shift_over_12dx(G, beta, bs);
    R db[3][3];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) db[i][j] = d1ptr(d1, G, nfield, j, MIX_B + i, p)[0];
    const R div = db[0][0] + db[1][1] + db[2][2];
    R Au[6];  // A^ij = g^ik (g^jl A_lk)
    {
        R M[3][3];  // M[k][j] = g^kl A_lj
#pragma unroll
        for (int kk = 0; kk < 3; ++kk)
#pragma unroll
            for (int j = 0; j < 3; ++j)
                M[kk][j] = gi[sym(kk, 0)] * A[sym(0, j)] + gi[sym(kk, 1)] * A[sym(1, j)] + gi[sym(kk, 2)] * A[sym(2, j)];
        const R aK = alpha * K, m2a = R(-2.0) * alpha, m23div = R(-2.0 / 3.0) * div;
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int j = i; j < 3; ++j) {
                R AgA = R(0), lie = R(0);
#pragma unroll
                for (int kk = 0; kk < 3; ++kk) {
                    AgA += A[sym(i, kk)] * M[kk][j];
                    lie += A[sym(kk, i)] * db[kk][j] + A[sym(kk, j)] * db[kk][i];
                }
                const int s = sym(i, j);
                T[s] = (aK * A[s] + m2a * AgA) + T[s] + lie + m23div * A[s];
                Au[s] = gi[sym(i, 0)] * M[j][0] + gi[sym(i, 1)] * M[j][1] + gi[sym(i, 2)] * M[j][2];
            }
    }
    // dt At_ij (extrinsic_curvature.py:100-175)
#pragma unroll 1
    for (int s = 0; s < 6; ++s) {
        const R* f = u + (AXX + s) * cs + p;
        R v = T[s] + ADV<R, Closed, false>(f, G, c.ix, beta, bs);
        if (damp != nullptr) v += damp[s * cs + p];
        k[(AXX + s) * cs + p] = v + KO<R, Closed, false>(f, G, c.ix);
    }
    // dt K (extrinsic_curvature.py:20-87)
    {
        const R* f = u + CK * cs + p;
        R bulk = -lapse_lap + alpha * contract_sym(A, Au) + alpha * (K * K) / R(3.0)
                 + ADV<R, Closed, false>(f, G, c.ix, beta, bs);
        if (mat != nullptr) {
            const R wf = static_cast<R>(fmax(u64[CW * cs + p], 1.0e-12));
            const R wf2 = wf * wf;
            R trace = R(0);
#pragma unroll
            for (int i = 0; i < 3; ++i)
#pragma unroll
                for (int j = 0; j < 3; ++j) trace += (wf2 * gi[sym(i, j)]) * static_cast<R>(mat[(4 + sym(i, j)) * cs + p]);
            bulk = bulk + R(4.0 * kPi) * alpha * (static_cast<R>(mat[p]) + trace);
        }
        k[CK * cs + p] = bulk + KO<R, Closed, false>(f, G, c.ix);
    }
    // dt Gt^i (conformal_connection.py:20-178)
    R dK[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) dK[d] = D1<R, Closed>(u + CK * cs + p, G, d, c.ix[d]);
    R six_alpha_over_w;
    if constexpr (kPerturbative<R>) {
        six_alpha_over_w = R(-6.0) * alpha * static_cast<R>(1.0 / fmax(u64[CW * cs + p], 1.0e-12));
    } else {
        const R Wf = fmax(W, 1.0e-12);
        six_alpha_over_w = -6.0 * alpha / Wf;
    }
    R hb[3][6];  // hb[i][sym(m,n)] = d_m d_n beta^i
#pragma unroll 1
    for (int i = 0; i < 3; ++i) hessian<R, Closed, kExactBg<R>>(u, d1, G, nfield, BX + i, MIX_B + i, c, hb[i]);
    R graddiv[3];
#pragma unroll
    for (int m = 0; m < 3; ++m) graddiv[m] = hb[0][sym(m, 0)] + hb[1][sym(m, 1)] + hb[2][sym(m, 2)];
    const R Gt[3] = {full(u, GTX, G, c), full(u, GTY, G, c), full(u, GTZ, G, c)};
#pragma unroll 1
    for (int i = 0; i < 3; ++i) {
        R t1 = R(0), t3 = R(0), t4 = R(0), t7 = R(0), t9 = R(0);
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            t1 += gi[sym(i, j)] * dK[j];
            t3 += Au[sym(i, j)] * dW[j];
            t4 += Au[sym(i, j)] * da[j];
            t7 += Gt[j] * db[i][j];
            t9 += gi[sym(i, j)] * graddiv[j];
        }
        const R t2 = contract_sym(c2[i], Au);
        const R t8 = contract_sym(gi, hb[i]);
        const R* f = u + (GTX + i) * cs + p;
        const R v = R(-4.0 / 3.0) * alpha * t1 + R(2.0) * alpha * t2 + six_alpha_over_w * t3
                    - R(2.0) * t4 + ADV<R, Closed, false>(f, G, c.ix, beta, bs) + R(2.0 / 3.0) * Gt[i] * div - t7 + t8
                    + R(1.0 / 3.0) * t9;
        R out = v + KO<R, Closed, false>(f, G, c.ix);
        if (mat != nullptr) {
            R gs = R(0);
#pragma unroll
            for (int j = 0; j < 3; ++j) gs += gi[sym(i, j)] * static_cast<R>(mat[(1 + j) * cs + p]);
            out = out + R(-16.0 * kPi) * alpha * gs;
        }
        k[(GTX + i) * cs + p] = out;
    }
}

// ---------------------------------------------------------------------------
// kappa != 0: pointwise derived fields (constraints.py:112-118):
//   der[0..5]  = gt^ij        der[6..14] = B_i^j = gt^jk At_ik
//   der[15..23]= B_i^j / max(W, 1e-12)
// ---------------------------------------------------------------------------
template <typename R>
__global__ void __launch_bounds__(kThreads)
k_mom_derived(const R* __restrict__ u, const double* __restrict__ u64, R* __restrict__ der, Geo G, Box all) {
    PointCtx c;
    if (!point(all, c, G)) return;
    const long long cs = G.cs, p = c.p;
    R g[6], gi[6], A[6];
    load_sym(u, GXX, G, c, g);
    load_sym(u, AXX, G, c, A);
    inverse_metric(g, gi);
    R inv_w;
    if constexpr (kPerturbative<R>) inv_w = static_cast<R>(1.0 / fmax(u64[CW * cs + p], 1.0e-12));
#pragma unroll
    for (int s = 0; s < 6; ++s) der[s * cs + p] = gi[s];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            const R b = gi[sym(j, 0)] * A[sym(i, 0)] + gi[sym(j, 1)] * A[sym(i, 1)] + gi[sym(j, 2)] * A[sym(i, 2)];
            der[(6 + 3 * i + j) * cs + p] = b;
            if constexpr (kPerturbative<R>) {
                der[(15 + 3 * i + j) * cs + p] = b * inv_w;
            } else {
                const R Wf = fmax(u[CW * cs + p], 1.0e-12);
                der[(15 + 3 * i + j) * cs + p] = b / Wf;
            }
        }
}

// kappa/2 alpha (D_j M_i + D_i M_j) into damp[6] (extrinsic_curvature.py:390-404)
template <typename R, bool Closed>
__global__ void __launch_bounds__(kThreads)
k_mom_damping(const R* __restrict__ u, const double* __restrict__ u64, const R* __restrict__ der,
              const R* __restrict__ d1, const double* __restrict__ mat, R* __restrict__ damp, Geo G, BoxSet S,
              int nfield) {
    PointCtx c;
    if (!point<Closed>(S.b[blockIdx.y], c, G)) return;
    const long long cs = G.cs, p = c.p;
    const int fA = NMIX, fK = NMIX + 6, fB = NMIX + 7;
    R gi[6];
#pragma unroll
    for (int s = 0; s < 6; ++s) gi[s] = der[s * cs + p];
    R three_over_w;  // 3 / max(W, 1e-12), from the FP64 state in the FP32 form
    if constexpr (kPerturbative<R>) three_over_w = static_cast<R>(3.0 / fmax(u64[CW * cs + p], 1.0e-12));
    R dW[3], dK[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        dW[d] = d1ptr(d1, G, nfield, d, MIX_W, p)[0];
        dK[d] = d1ptr(d1, G, nfield, d, fK, p)[0];
    }
    // M_i (constraints.py:61-97)
    R M[3];
#pragma unroll 1
    for (int i = 0; i < 3; ++i) {
        R first = R(0), second = R(0), third = R(0);
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            first += d1ptr(d1, G, nfield, j, fB + 3 * i + j, p)[0];
            third += der[(6 + 3 * i + j) * cs + p] * dW[j];
        }
#pragma unroll
        for (int s = 0; s < 6; ++s) {
            const R w = (s == 0 || s == 3 || s == 5) ? R(1.0) : R(2.0);
            second += w * gi[s] * d1ptr(d1, G, nfield, i, fA + s, p)[0];
        }
        if constexpr (kPerturbative<R>) {
            M[i] = first - R(0.5) * second - third * three_over_w - R(2.0 / 3.0) * dK[i];
        } else {
            const R Wf = fmax(u[CW * cs + p], 1.0e-12);
            M[i] = first - 0.5 * second - 3.0 * third / Wf - (2.0 / 3.0) * dK[i];
        }
    }
    // d_l M_i (constraints.py:186-213), dM[i][l]
    R hW[6];
    hessian<R, Closed, kExactBg<R>>(u, d1, G, nfield, CW, MIX_W, c, hW);
    R dM[3][3];
#pragma unroll 1
    for (int i = 0; i < 3; ++i) {
#pragma unroll 1
        for (int l = 0; l < 3; ++l) {
            R divd = R(0), conf = R(0), met = R(0), met2 = R(0);
#pragma unroll 1
            for (int j = 0; j < 3; ++j) {
                // d_l d_j B_ij
                const int fb = fB + 3 * i + j;
                divd += (l == j) ? D2<R, Closed, false>(der + (6 + 3 * i + j) * cs + p, G, l, c.ix[l])
                                 : mixed<R, Closed>(d1, G, nfield, fb, l, j, c);
                const R dBW = D1<R, Closed>(der + (15 + 3 * i + j) * cs + p, G, l, c.ix[l]);
                conf += dBW * dW[j] + der[(15 + 3 * i + j) * cs + p] * hW[sym(l, j)];
            }
#pragma unroll 1
            for (int s = 0; s < 6; ++s) {
                const R w = (s == 0 || s == 3 || s == 5) ? R(1.0) : R(2.0);
                const R dgi = D1<R, Closed>(der + s * cs + p, G, l, c.ix[l]);
                met += w * dgi * d1ptr(d1, G, nfield, i, fA + s, p)[0];
                const R d2A = (l == i) ? D2<R, Closed, false>(u + (AXX + s) * cs + p, G, l, c.ix[l])
                                       : mixed<R, Closed>(d1, G, nfield, fA + s, l, i, c);
                met2 += w * gi[s] * d2A;
            }
            const R d2K = (l == i) ? D2<R, Closed, false>(u + CK * cs + p, G, l, c.ix[l]) : mixed<R, Closed>(d1, G, nfield, fK, l, i, c);
            dM[i][l] = divd - R(0.5) * met - R(0.5) * met2 - R(3.0) * conf - R(2.0 / 3.0) * d2K;
        }
    }
    if (mat != nullptr) {
        // matter momentum: M_i - 8 pi S_i, d_l M_i - 8 pi d_l S_i (constraints.py:233-259)
#pragma unroll 1
        for (int i = 0; i < 3; ++i) {
            const double* Sp = mat + (1 + i) * cs + p;
            M[i] = M[i] - R(8.0 * kPi) * static_cast<R>(Sp[0]);
#pragma unroll 1
            for (int l = 0; l < 3; ++l)
                dM[i][l] = dM[i][l] - R(8.0 * kPi) * static_cast<R>(D1<double, Closed>(Sp, G, l, c.ix[l]));
        }
    }
    // Christoffels for D_j M_i = d_j M_i - Gamma^k_ij M_k
    R g[6], gl[6];
    load_sym(u, GXX, G, c, g);
    inverse_metric(g, gl);
    R c1[3][6], c2[3][6];
    {
        R dg[3][6];
        load_metric_derivs(d1, G, nfield, p, dg);
        christoffel(dg, gl, c1, c2);
    }
    const R scale = BSSN_CO(R, G, kappa) / R(2.0) * full_exact(u, u64, CALPHA, cs, p);
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = i; j < 3; ++j) {
            const int s = sym(i, j);
            const R gm = c2[0][s] * M[0] + c2[1][s] * M[1] + c2[2][s] * M[2];
            const R DjMi = dM[i][j] - gm;
            const R DiMj = dM[j][i] - gm;
            damp[s * cs + p] = scale * (DjMi + DiMj);
        }
}

// ---------------------------------------------------------------------------
// Sommerfeld faces: rhs = -(x^i/r d_i u + (u - u_inf)/r) (boundaries.py:74-147)
// In the FP32 form the stored perturbation is already u - u_inf.
// ---------------------------------------------------------------------------
// Sommerfeld replacement on one-sample slabs at the active faces; an edge
// sample in two slabs is computed twice with the same result.
constexpr int kSommerfeldGroup = 3;   // 7 groups of 3 components
static_assert(NCOMP % kSommerfeldGroup == 0, "component groups must tile the state");

template <typename R>
__global__ void __launch_bounds__(kThreads)
k_sommerfeld(const R* __restrict__ u, const double* __restrict__ u64, double* __restrict__ k, Geo G, BoxSet S) {
    PointCtx c;
    if (!point(S.b[blockIdx.y], c, G)) return;
    bool face = false;
    bool owned = true;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        const Axis& a = G.ax[d];
        owned = owned && c.ix[d] >= a.start && c.ix[d] < a.end;
        face = face || (a.slo && c.ix[d] == a.start) || (a.shi && c.ix[d] == a.end - 1);
    }
    if (!(face && owned)) return;
    R xr[3], rr;
    if constexpr (kPerturbative<R>) {
        // float forms: the radial direction in float (FP64 arithmetic runs
        // at a small fraction of the float rate here, and these values end
        // up in float anyway)
        float r2 = 0.0f;
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            xr[d] = static_cast<float>(G.ax[d].xmin) + static_cast<float>(G.dx) * (float)(c.ix[d] - G.ax[d].org);
            r2 += xr[d] * xr[d];
        }
        const float r = sqrtf(r2);
        rr = r > 0.0f ? r : 1.0f;
    } else {
        // FP64 form: the reference's operation order
        double X[3];
#pragma unroll
        for (int d = 0; d < 3; ++d) X[d] = __dadd_rn(G.ax[d].xmin, __dmul_rn(G.dx, (double)(c.ix[d] - G.ax[d].org)));
        const double r = __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(X[0], X[0]), __dmul_rn(X[1], X[1])),
                                              __dmul_rn(X[2], X[2])));
#pragma unroll
        for (int d = 0; d < 3; ++d) xr[d] = X[d];
        rr = r > 0.0 ? r : 1.0;
    }
    const long long cs = G.cs, p = c.p;
    // blockIdx.z picks a group of kSommerfeldGroup components: short per-thread
    // chains and enough threads for the few face samples
#pragma unroll 1
    for (int comp = blockIdx.z * kSommerfeldGroup; comp < (int)(blockIdx.z + 1) * kSommerfeldGroup; ++comp) {
        const R* f = u + comp * cs + p;
        const R radial = (xr[0] * D1<R, true>(f, G, 0, c.ix[0]) + xr[1] * D1<R, true>(f, G, 1, c.ix[1])
                          + xr[2] * D1<R, true>(f, G, 2, c.ix[2])) / rr;
        R offset;
        if constexpr (kPerturbative<R>) {
            offset = static_cast<R>(u64[comp * cs + p] - (has_background(comp) ? 1.0 : 0.0));
        } else {
            const R asym = has_background(comp) ? 1.0 : 0.0;
            offset = f[0] - asym;
        }
        k[comp * cs + p] = -(radial + offset / rr);
    }
}

// ---------------------------------------------------------------------------
// Constraint fields (JAX_BSSN/bssn/constraints.py:22-97, 271-412): H, M_i,
// det(gt) - 1, gt^ij At_ij and Gt^i - gt^jk Gamma^i_jk, written in the
// reference layout at the box's linear index.  FP64 only.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kThreads)
k_constraints(const double* __restrict__ u, const double* __restrict__ d1, const double* __restrict__ der,
              Geo G, Box B, double* __restrict__ H, double* __restrict__ Mo, double* __restrict__ detm1,
              double* __restrict__ trA, double* __restrict__ gam) {
    PointCtx c;
    if (!point(B, c, G)) return;
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long n = B.count;
    const long long cs = G.cs, p = c.p;
    double g[6], gi[6], A[6];
    load_sym(u, GXX, G, c, g);
    load_sym(u, AXX, G, c, A);
    inverse_metric(g, gi);
    double c1[3][6], c2[3][6];
    {
        double dg[3][6];
        load_metric_derivs(d1, G, NMIX, p, dg);
        christoffel(dg, gi, c1, c2);
    }
    double dW[3], dK[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        dW[d] = d1ptr(d1, G, NMIX, d, MIX_W, p)[0];
        dK[d] = D1<double, true>(u + CK * cs + p, G, d, c.ix[d]);
    }
    const double W = u[CW * cs + p];
    const double K = u[CK * cs + p];
    double w2r[6];
    w2_ricci<double, true>(u, d1, G, NMIX, c, g, gi, c1, c2, dW, W, w2r);
    double Au[6];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = i; j < 3; ++j) {
            double acc = 0.0;
#pragma unroll
            for (int kk = 0; kk < 3; ++kk)
#pragma unroll
                for (int l = 0; l < 3; ++l) acc += gi[sym(i, kk)] * gi[sym(j, l)] * A[sym(kk, l)];
            Au[sym(i, j)] = acc;
        }
    H[t] = contract_sym(gi, w2r) + 2.0 / 3.0 * (K * K) - contract_sym(A, Au);
    const double Wf = fmax(W, 1.0e-12);
#pragma unroll 1
    for (int i = 0; i < 3; ++i) {
        double first = 0.0, second = 0.0, third = 0.0;
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            first += D1<double, true>(der + (6 + 3 * i + j) * cs + p, G, j, c.ix[j]);
            third += der[(6 + 3 * i + j) * cs + p] * dW[j];
        }
#pragma unroll 1
        for (int s = 0; s < 6; ++s) {
            const double w = (s == 0 || s == 3 || s == 5) ? 1.0 : 2.0;
            second += w * gi[s] * D1<double, true>(u + (AXX + s) * cs + p, G, i, c.ix[i]);
        }
        Mo[i * n + t] = first - 0.5 * second - 3.0 * third / Wf - (2.0 / 3.0) * dK[i];
        gam[i * n + t] = u[(GTX + i) * cs + p] - contract_sym(gi, c2[i]);
    }
    detm1[t] = det_sym_rn(g) - 1.0;
    trA[t] = contract_sym(gi, A);
}

// The box grown by `by` samples on every side, clipped to the padded block.
static Box grown_box(const Box& box, const Geo& G, int by) {
    Box b;
    b.count = 1;
    for (int d = 0; d < 3; ++d) {
        // An axis whose two owned faces are Sommerfeld-closed and which the box
        // spans is not grown: its closures cover the three outer rows and every
        // interior stencil stays inside the owned samples, so nothing beyond
        // them is read.
        const Axis& a = G.ax[d];
        const bool closed = !a.reduced && a.lbc && a.rbc && box.lo[d] == a.start && box.lo[d] + box.n[d] == a.end;
        const int g = closed ? 0 : by;
        int lo = box.lo[d] - g, hi = box.lo[d] + box.n[d] + g;
        if (lo < 0) lo = 0;
        if (hi > G.ax[d].P) hi = G.ax[d].P;
        b.lo[d] = lo;
        b.n[d] = hi - lo;
        b.count *= b.n[d];
    }
    return b;
}

// First derivatives are needed on the box grown by the reach of the
// second-derivative composition (D1 of D1): 2 samples, 3 with MAD weights.
static int composition_reach(const Geo& G) {
    int reach = 2;
    for (int d = 0; d < 3; ++d) if (G.ax[d].mad) reach = 3;
    return reach;
}

static inline unsigned blocks_for(long long n) { return (unsigned)((n + kThreads - 1) / kThreads); }

static Box make_box(const int lo[3], const int hi[3], int fast = 2) {
    Box b;
    b.fast = fast;
    b.count = 1;
    for (int d = 0; d < 3; ++d) {
        b.lo[d] = lo[d];
        b.n[d] = hi[d] > lo[d] ? hi[d] - lo[d] : 0;
        b.count *= b.n[d];
    }
    return b;
}

static void add_box(BoxSet& S, const Box& b) {
    if (b.count > 0) S.b[S.n++] = b;
}

static long long largest(const BoxSet& S) {
    long long m = 0;
    for (int i = 0; i < S.n; ++i) m = S.b[i].count > m ? S.b[i].count : m;
    return m;
}

// Block size of a box-set launch: kThreads, or fewer (down to one warp) when
// kThreads would leave under four blocks per SM.  With GB300's two FP64 lanes
// per SM per cycle, a small launch (a Cartoon plane, the shell of a small box)
// otherwise runs a few FP64-heavy blocks on a few SMs while the rest idle.
static inline int set_threads(const BoxSet& S, int ninst) {
    long long total = 0;
    for (int i = 0; i < S.n; ++i) total += S.b[i].count * ninst;
    for (int t = kThreads; t > 32; t /= 2)
        if ((total + t - 1) / t >= 152LL * 4) return t;
    return 32;
}

// A box split into its interior -- samples at least kClosureRows from every
// closed (Sommerfeld) owned face, where no stencil needs a one-sided closure --
// and the rest of the box as up to ten slabs.
struct SplitBox {
    BoxSet interior, shell;
};

static SplitBox split_box(const Geo& G, const Box& box, bool coalesced) {
    int blo[3], bhi[3], lo[3], hi[3];
    for (int d = 0; d < 3; ++d) {
        const Axis& a = G.ax[d];
        blo[d] = box.lo[d];
        bhi[d] = box.lo[d] + box.n[d];
        lo[d] = blo[d];
        hi[d] = bhi[d];
        if (a.lbc && !a.reduced) lo[d] = lo[d] > a.start + kClosureRows ? lo[d] : a.start + kClosureRows;
        if (a.rbc && !a.reduced) hi[d] = hi[d] < a.end - kClosureRows ? hi[d] : a.end - kClosureRows;
        if (lo[d] > bhi[d]) lo[d] = bhi[d];
        if (hi[d] < lo[d]) hi[d] = lo[d];
    }
    SplitBox S;
    S.interior.n = 0;
    S.shell.n = 0;
    add_box(S.interior, make_box(lo, hi));
    if (coalesced) {
        // z fastest everywhere (coalesced loads, for the load-bound FP32
        // form): x slabs over the whole box in y and z, y slabs inside x, z
        // slabs inside x and y.
        for (int d = 0; d < 3; ++d) {
            int l0[3], h0[3], l1[3], h1[3];
            for (int e = 0; e < 3; ++e) {
                const bool inner = e < d;   // axes already sliced take the interior range
                l0[e] = l1[e] = inner ? lo[e] : blo[e];
                h0[e] = h1[e] = inner ? hi[e] : bhi[e];
            }
            l0[d] = blo[d]; h0[d] = lo[d];
            l1[d] = hi[d];  h1[d] = bhi[d];
            add_box(S.shell, make_box(l0, h0));
            add_box(S.shell, make_box(l1, h1));
        }
        return S;
    }
    // The shell (for the FP64 form, bound by FP64 instructions), cut so that the fast axis of every slab runs through the
    // interior range of its axis: the 32 samples of a warp then share their
    // closure rows (no divergent closure branches), except where a warp wraps
    // to the next row.
    //   z rows:  z in the closure rows, y interior, x whole box; y fastest,
    //            or x fastest when the y range is shorter than a warp and
    //            than the x range (a single-plane Cartoon box)
    //   y rows:  y in the closure rows, z interior, x whole box; z fastest
    //   yz rows: y and z in the closure rows, x whole box; x fastest
    //   x rows:  x in the closure rows, y and z interior; z fastest
    const int E0[2] = {blo[0], hi[0]}, E1[2] = {lo[0], bhi[0]};  // x closure ranges [E0, E1)
    const int Y0[2] = {blo[1], hi[1]}, Y1[2] = {lo[1], bhi[1]};
    const int Z0[2] = {blo[2], hi[2]}, Z1[2] = {lo[2], bhi[2]};
    const int ny = hi[1] - lo[1], nx = bhi[0] - blo[0];
    const int zrow_fast = (ny >= 32 || ny >= nx) ? 1 : 0;
    for (int f = 0; f < 2; ++f) {
        const int l[3] = {blo[0], lo[1], Z0[f]}, h[3] = {bhi[0], hi[1], Z1[f]};
        add_box(S.shell, make_box(l, h, zrow_fast));
    }
    for (int f = 0; f < 2; ++f) {
        const int l[3] = {blo[0], Y0[f], lo[2]}, h[3] = {bhi[0], Y1[f], hi[2]};
        add_box(S.shell, make_box(l, h, 2));
    }
    for (int f = 0; f < 2; ++f)
        for (int e = 0; e < 2; ++e) {
            const int l[3] = {blo[0], Y0[f], Z0[e]}, h[3] = {bhi[0], Y1[f], Z1[e]};
            add_box(S.shell, make_box(l, h, 0));
        }
    for (int f = 0; f < 2; ++f) {
        const int l[3] = {E0[f], lo[1], lo[2]}, h[3] = {E1[f], hi[1], hi[2]};
        add_box(S.shell, make_box(l, h, 2));
    }
    return S;
}

static BoxSet single(const Box& b) {
    BoxSet S;
    S.n = 0;
    add_box(S, b);
    return S;
}

// The box's samples on each active Sommerfeld face (owned face index on that
// axis, the box's range on the others).
// The box without its samples on active Sommerfeld face planes (the planes
// face_slabs lists).
static Box without_faces(const Geo& G, const Box& box) {
    int lo[3], hi[3];
    for (int d = 0; d < 3; ++d) {
        const Axis& a = G.ax[d];
        lo[d] = box.lo[d];
        hi[d] = box.lo[d] + box.n[d];
        if (a.slo && lo[d] == a.start && lo[d] < hi[d]) ++lo[d];
        if (a.shi && hi[d] == a.end && hi[d] > lo[d]) --hi[d];
    }
    return make_box(lo, hi);
}

static BoxSet face_slabs(const Geo& G, const Box& box) {
    BoxSet S;
    S.n = 0;
    for (int d = 0; d < 3; ++d) {
        const Axis& a = G.ax[d];
        const int faces[2] = {a.slo ? a.start : -1, a.shi ? a.end - 1 : -1};
        for (int f = 0; f < 2; ++f) {
            const int i = faces[f];
            if (i < 0 || i < box.lo[d] || i >= box.lo[d] + box.n[d]) continue;
            if (f == 1 && a.slo && i == a.start) continue;   // one-sample axis: same slab
            Box b = box;
            b.lo[d] = i;
            b.n[d] = 1;
            b.count = (long long)b.n[0] * b.n[1] * b.n[2];
            S.b[S.n++] = b;
        }
    }
    return S;
}

// ---------------------------------------------------------------------------
// Launch-shape autotuning.  A box-set launch belongs to a slot -- its kernel
// class and whether it is the interior or the shell instantiation -- and
// takes its block size from the tuning table when bssn_tune_patch has timed
// that slot at that launch size on this device in this arithmetic form, else
// from the set_threads heuristic.  Tuning times whole RHS evaluations with
// each candidate block size for one slot at a time (coordinate descent) and
// keeps the fastest; only the launch shape changes, so results are identical
// bit for bit.
// ---------------------------------------------------------------------------
constexpr int kTuneCandidates[3] = {32, 64, 128};

struct TuneKey {
    int dev, cls, shell, precision;
    long long size;
    bool operator<(const TuneKey& o) const {
        if (dev != o.dev) return dev < o.dev;
        if (cls != o.cls) return cls < o.cls;
        if (shell != o.shell) return shell < o.shell;
        if (precision != o.precision) return precision < o.precision;
        return size < o.size;
    }
};

static std::mutex g_tune_lock;
static std::map<TuneKey, int> g_tuned;
// while tuning (on the tuning thread): the slot under test, its forced block
// size, and the launch size the slot was seen with
static thread_local int t_force_cls = -1, t_force_shell = -1, t_force_threads = 0;
static thread_local long long t_seen_size = -1;

static int launch_threads(int cls, int shell, const BoxSet& S, const Geo& G) {
    long long total = 0;
    for (int i = 0; i < S.n; ++i) total += S.b[i].count * G.ninst;
    if (cls == t_force_cls && shell == t_force_shell) {
        t_seen_size = total;
        return t_force_threads;
    }
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        cudaGetLastError();
        return set_threads(S, G.ninst);
    }
    {
        std::lock_guard<std::mutex> guard(g_tune_lock);
        if (!g_tuned.empty()) {
            const auto it = g_tuned.find(TuneKey{dev, cls, shell, G.precision, total});
            if (it != g_tuned.end()) return it->second;
        }
    }
    return set_threads(S, G.ninst);
}

// Launch over a box set; the launch's geometry must be in scope as G (its
// instance count multiplies the threads).  shell: 1 for the general (shell)
// instantiation, 0 for the closure-free interior one.
#define BSSN_LAUNCH_SET(cls, shell, kernel, set, stream, ...)                                              \
    do {                                                                                                  \
        if ((set).n > 0) {                                                                                \
            const int threads_ = launch_threads(cls, shell, set, G);                                      \
            const long long cover_ = largest(set) * G.ninst;                                              \
            BSSN_LAUNCH(cls, kernel, dim3((unsigned)((cover_ + threads_ - 1) / threads_), (set).n),         \
                        threads_, stream, __VA_ARGS__);                                                    \
        }                                                                                                 \
    } while (0)

cudaError_t launch_constraints(const double* u, const RhsWork& w, const Geo& G, const Box& box, double* H,
                               double* M, double* detm1, double* trA, double* gam, cudaStream_t stream) {
    const Box ext = grown_box(box, G, composition_reach(G));
    // derived fields are pointwise and read on the box only
    BSSN_LAUNCH(KC_MOM_DERIVED, k_mom_derived<double>, blocks_for(box_threads(G, ext)), kThreads, stream, u, u, w.der,
                G, ext);
    const BoxSet es = single(ext);
    BSSN_LAUNCH_SET(KC_FIRST, 1, (k_first_derivs<double, true>), es, stream, u, w.der, w.d1, G, es, 0);
    BSSN_LAUNCH(KC_CONSTRAINTS, k_constraints, blocks_for(box.count), kThreads, stream, u, w.d1, w.der, G, box,
                H, M, detm1, trA, gam);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Independent RHS kernels run on two auxiliary streams (per device and host
// thread), forked from and joined back to the caller's stream with events, so
// the block scheduler can fill one kernel's tail with another's blocks; under
// stream capture the forks become parallel graph branches.  Per-kernel
// profiling times each launch on its own, so it runs them serially; so does a
// call that is already being captured before the streams exist (creating them
// is not a capturable operation).
// ---------------------------------------------------------------------------
struct RhsStreams {
    cudaStream_t b = nullptr, c = nullptr;
    cudaEvent_t fork = nullptr, pre = nullptr, fd = nullptr, d1 = nullptr, join_b = nullptr, join_c = nullptr;
};

static RhsStreams* rhs_streams(cudaStream_t s) {
    if (profiling_enabled()) return nullptr;
    thread_local std::map<int, RhsStreams> all;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    auto it = all.find(dev);
    if (it != all.end()) return &it->second;
    cudaStreamCaptureStatus status = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(s, &status) != cudaSuccess || status != cudaStreamCaptureStatusNone) {
        cudaGetLastError();
        return nullptr;
    }
    RhsStreams X;
    bool ok = cudaStreamCreateWithFlags(&X.b, cudaStreamNonBlocking) == cudaSuccess &&
              cudaStreamCreateWithFlags(&X.c, cudaStreamNonBlocking) == cudaSuccess;
    for (cudaEvent_t* e : {&X.fork, &X.pre, &X.fd, &X.d1, &X.join_b, &X.join_c})
        ok = ok && cudaEventCreateWithFlags(e, cudaEventDisableTiming) == cudaSuccess;
    if (!ok) {
        cudaGetLastError();
        return nullptr;
    }
    return &(all[dev] = X);
}

// ---------------------------------------------------------------------------
// Host side of the TMA gauge kernel: the tensor map (cuTensorMapEncodeTiled,
// reached through the runtime's driver entry point), the per-device shared
// memory opt-in, and the geometry it serves -- z pitch a multiple of four
// floats (the box's z origin must sit on a 16-byte boundary), no MAD or
// reduced axis; batches are the tensor's fourth dimension.  Anything else
// takes k_rhs_gauge.
// ---------------------------------------------------------------------------
namespace {
using EncodeTiled = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                 const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                 CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
EncodeTiled encode_tiled() {
    static const EncodeTiled fn = [] {
        void* ptr = nullptr;
        cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &ptr, 12000, cudaEnableDefault, &q) !=
                cudaSuccess || q != cudaDriverEntryPointSuccess)
            return static_cast<EncodeTiled>(nullptr);
        return reinterpret_cast<EncodeTiled>(ptr);
    }();
    return fn;
}
// default: all four.  At 128^3 the FP32 step took 8.60 ms with the
// derivatives alone, 8.13 with the At kernel, 7.77 with the K/Gt kernel,
// 7.34 with the gauge kernel, 7.18 with the rows next to the Sommerfeld
// faces in the boxes, 6.93 once those rows share the centred taps, 6.90
// with the At kernel's spills cut and 6.79 with the first derivatives over the
// whole box (paired: 10.12, 9.43, 9.01, 8.57, 8.35, 8.09, 8.05, 7.85 ms).  A gauge
// kernel with four samples per thread and 90 KB of shared memory per CTA was
// faster alone but crowded out the kernels beside it (9.55 against 9.42 ms).
std::atomic<int> g_tma_mask{kTmaAll};
std::atomic<long long> g_tma_launches{0};
__device__ int g_tma_timeouts;

// per device: shared-memory opt-in done, and the timeout counter's address
struct TmaDevice {
    bool ready = false;
    int* timeouts = nullptr;
};
cudaError_t tma_device(TmaDevice& out) {
    static std::mutex lock;
    static std::map<int, TmaDevice> devices;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    std::lock_guard<std::mutex> guard(lock);
    TmaDevice& d = devices[dev];
    if (!d.ready) {
        e = cudaFuncSetAttribute(k_rhs_gauge_tma, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)tma::curv_smem(0));
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(k_first_derivs_tma<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)tma::DSMEM);
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(k_first_derivs_tma<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)tma::DSMEM);
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(k_rhs_at_tma, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)tma::curv_smem(tma::AT_NQ));
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(k_rhs_kgt_tma, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)tma::curv_smem(tma::KGT_NQ));
        if (e == cudaSuccess) e = cudaGetSymbolAddress(reinterpret_cast<void**>(&d.timeouts), g_tma_timeouts);
        if (e != cudaSuccess) return e;
        d.ready = true;
    }
    out = d;
    return cudaSuccess;
}
}  // namespace

void set_tma_kernels(int mask) { g_tma_mask.store(mask & kTmaAll); }

long long tma_launches() { return g_tma_launches.load(); }

cudaError_t tma_timeouts(int* count) {
    int zero = 0;
    cudaError_t e = cudaMemcpyFromSymbol(count, g_tma_timeouts, sizeof(int));
    if (e == cudaSuccess) e = cudaMemcpyToSymbol(g_tma_timeouts, &zero, sizeof(int));
    return e;
}

// The interior first derivatives of the FP32 forms from TMA tiles (kappa = 0:
// the NMIX fields only); false leaves the launch to the generic kernel.
// closed: S may hold the D1 closure rows next to Sommerfeld faces (the whole
// box, on a grid where tma_whole_box holds).
static bool launch_first_derivs_tma(const float* u, float* d1, const Geo& G, const BoxSet& S, int with_mom,
                                    bool closed, cudaStream_t stream) {
    if (!(g_tma_mask.load() & kTmaDerivs) || with_mom || S.n != 1 || G.ninst < 1 || G.ninst > 65535) return false;
    for (int d = 0; d < 3; ++d)
        if (G.ax[d].mad || G.ax[d].reduced) return false;
    if (G.ax[2].P % 4 != 0 || reinterpret_cast<uintptr_t>(u) % 16 != 0 || reinterpret_cast<uintptr_t>(d1) % 16 != 0)
        return false;
    const EncodeTiled encode = encode_tiled();
    if (!encode) return false;
    TmaDevice dev;
    if (tma_device(dev) != cudaSuccess) return false;
    const Box& B = S.b[0];
    const long long istride = G.istride;
    // (z, y, x, instance, component): the 21 perturbations and the 11 low words
    const cuuint64_t dims[5] = {(cuuint64_t)G.ax[2].P, (cuuint64_t)G.ax[1].P, (cuuint64_t)G.ax[0].P,
                                (cuuint64_t)G.ninst, (cuuint64_t)(NCOMP + NMIX)};
    const cuuint64_t strides[4] = {(cuuint64_t)G.st[1] * 4, (cuuint64_t)G.st[0] * 4, (cuuint64_t)istride * 4,
                                   (cuuint64_t)G.cs * 4};
    const cuuint32_t box[5] = {tma::DHZ, tma::DHY, tma::DHX, 1, 1};
    const cuuint32_t unit[5] = {1, 1, 1, 1, 1};
    if (istride * 4 % 16 != 0) return false;
    CUtensorMap map;
    if (encode(&map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 5, const_cast<float*>(u), dims, strides, box, unit,
               CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
        return false;
    const int z_base = B.lo[2] & ~3;
    const int tiles_z = (B.lo[2] + B.n[2] - z_base + tma::TZ - 1) / tma::TZ;
    const int tiles_y = (B.n[1] + tma::TY - 1) / tma::TY;
    const int tiles_x = (B.n[0] + tma::TX - 1) / tma::TX;
    const long long tiles = (long long)tiles_z * tiles_y * tiles_x;
    if (tiles <= 0 || tiles > 0x7fffffffLL) return false;
    const int paired = G.precision == kPrecisionF32Paired ? 1 : 0;
    prof_begin(KC_FIRST, stream);
    if (closed)
        k_first_derivs_tma<true><<<dim3((unsigned)tiles, (unsigned)G.ninst), tma::THREADS, tma::DSMEM, stream>>>(
            map, d1, G, B, z_base, tiles_z, tiles_y, NMIX, paired, dev.timeouts);
    else
        k_first_derivs_tma<false><<<dim3((unsigned)tiles, (unsigned)G.ninst), tma::THREADS, tma::DSMEM, stream>>>(
            map, d1, G, B, z_base, tiles_z, tiles_y, NMIX, paired, dev.timeouts);
    prof_end(KC_FIRST, stream);
    g_tma_launches.fetch_add(1);
    return true;
}

// Whether the TMA box kernels can take the whole box minus its face planes:
// every axis either without closures (periodic, the box's ghosts filled) or
// closed by Sommerfeld faces at both ends with the face condition active, the
// box spanning its owned samples and at least 16 of them (so that the rows
// next to the two faces never share a tile), and no MAD or reduced axis.
static bool tma_whole_box(const Geo& G, const Box& box) {
    if (!G.any_sommerfeld) return false;
    for (int d = 0; d < 3; ++d) {
        const Axis& a = G.ax[d];
        if (a.mad || a.reduced || a.lbc != a.rbc) return false;
        if (!a.lbc) continue;
        if (a.slo != 1 || a.shi != 1 || box.lo[d] != a.start || box.lo[d] + box.n[d] != a.end ||
            a.end - a.start < 16)
            return false;
    }
    return true;
}

// The interior RHS of the FP32 forms from TMA boxes: dt At (kc = KC_AT, mask
// bit kTmaAt) or dt K and dt Gt^i (KC_KGT, kTmaKgt), both for kappa = 0 in
// vacuum, or the gauge RHS (KC_GAUGE, kTmaGauge); false leaves the launch to
// the generic kernel.
static bool launch_curv_tma(int kc, const float* u, const double* u64, const float* d1, const float* damp,
                            const double* mat, double* k, const Geo& G, const BoxSet& S, int nfield,
                            cudaStream_t stream) {
    const int bit = kc == KC_AT ? kTmaAt : (kc == KC_KGT ? kTmaKgt : kTmaGauge);
    const bool curvature = kc != KC_GAUGE;
    if (!(g_tma_mask.load() & bit) || (curvature && (damp != nullptr || mat != nullptr || nfield != NMIX)) ||
        S.n != 1 || G.ninst < 1 || G.ninst > 65535)
        return false;
    for (int d = 0; d < 3; ++d)
        if (G.ax[d].mad || G.ax[d].reduced) return false;
    if (G.ax[2].P % 4 != 0 || reinterpret_cast<uintptr_t>(u) % 16 != 0 || reinterpret_cast<uintptr_t>(d1) % 16 != 0)
        return false;
    const long long istride = G.istride;
    if (istride * 4 % 16 != 0) return false;
    const EncodeTiled encode = encode_tiled();
    if (!encode) return false;
    TmaDevice dev;
    if (tma_device(dev) != cudaSuccess) return false;
    const Box& B = S.b[0];
    // (z, y, x, instance, component) over the FP32 state with its low words,
    // and over the first-derivative buffer (3 nfield components)
    const cuuint64_t strides[4] = {(cuuint64_t)G.st[1] * 4, (cuuint64_t)G.st[0] * 4, (cuuint64_t)istride * 4,
                                   (cuuint64_t)G.cs * 4};
    const cuuint32_t unit[5] = {1, 1, 1, 1, 1};
    tma::CurvMaps maps;
    for (int kind = 0; kind < 4; ++kind) {
        const bool state = kind == tma::kBoxV2 || kind == tma::kBoxV3;
        const cuuint64_t dims[5] = {(cuuint64_t)G.ax[2].P, (cuuint64_t)G.ax[1].P, (cuuint64_t)G.ax[0].P,
                                    (cuuint64_t)G.ninst, (cuuint64_t)(state ? NCOMP + NMIX : 3 * nfield)};
        const cuuint32_t box[5] = {(cuuint32_t)tma::AHZ, (cuuint32_t)tma::a_hy(kind), (cuuint32_t)tma::a_hx(kind), 1,
                                   1};
        void* base = state ? const_cast<float*>(u) : const_cast<float*>(d1);
        if (encode(&maps.map[kind], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 5, base, dims, strides, box, unit,
                   CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                   CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
            return false;
    }
    const int z_base = B.lo[2] & ~3;
    const int tiles_z = (B.lo[2] + B.n[2] - z_base + tma::AZ - 1) / tma::AZ;
    const int tiles_y = (B.n[1] + tma::AY - 1) / tma::AY;
    const int tiles_x = (B.n[0] + tma::AX - 1) / tma::AX;
    const long long tiles = (long long)tiles_z * tiles_y * tiles_x;
    if (tiles <= 0 || tiles > 0x7fffffffLL) return false;
    const int paired = G.precision == kPrecisionF32Paired ? 1 : 0;
    const dim3 grid((unsigned)tiles, (unsigned)G.ninst);
    prof_begin(kc, stream);
    if (kc == KC_AT)
        k_rhs_at_tma<<<grid, tma::A_THREADS, tma::curv_smem(tma::AT_NQ), stream>>>(
            maps, u, u64, d1, k, G, B, z_base, tiles_z, tiles_y, nfield, paired, dev.timeouts);
    else if (kc == KC_KGT)
        k_rhs_kgt_tma<<<grid, tma::A_THREADS, tma::curv_smem(tma::KGT_NQ), stream>>>(
            maps, u, u64, d1, k, G, B, z_base, tiles_z, tiles_y, nfield, paired, dev.timeouts);
    else
        k_rhs_gauge_tma<<<grid, tma::A_THREADS, tma::curv_smem(0), stream>>>(
            maps, u, u64, d1, k, G, B, z_base, tiles_z, tiles_y, nfield, paired, dev.timeouts);
    prof_end(kc, stream);
    g_tma_launches.fetch_add(1);
    return true;
}

// ---------------------------------------------------------------------------
// host-side launch sequence of one RHS evaluation: every stencil kernel runs
// as a closure-free instantiation on the box interior and a general one on
// the shell slabs.  Stream use (with the auxiliary streams b and c):
//   c: Sommerfeld face planes (reads only the state)
//   main: [momentum derived fields], first derivatives (interior); b: the
//      shell's first derivatives
//   b: gauge RHS (FP64) or K/Gt RHS and the shell's [momentum damping] and
//      At RHS (FP32); c: gauge RHS (FP32), or the shell's [momentum damping]
//      and K/Gt/At RHS (FP64)
//   main: the interior's [momentum damping] and K/Gt/At (FP64) or At (FP32)
// (the damping term enters the curvature RHS at its own point only).
// The stencil kernels skip the Sommerfeld face planes, and each writes its
// own components, so the branches write disjoint parts of k.
// ---------------------------------------------------------------------------
template <typename R>
static void launch_rhs_form(const R* u, const double* u64, double* k, R* d1, R* der, R* damp, const double* mat,
                            const Geo& G, const Box& box, cudaStream_t stream) {
    const int with_mom = G.kappa != 0.0;
    const int nfield = with_mom ? NMIX + NMIX_MOM : NMIX;
    const int reach = composition_reach(G);
    const Box ext = grown_box(box, G, reach);
    RhsStreams* X = rhs_streams(stream);
    const cudaStream_t stb = X ? X->b : stream, stc = X ? X->c : stream;
    if (X) {
        cudaEventRecord(X->fork, stream);
        cudaStreamWaitEvent(stc, X->fork, 0);
    }
    if (G.any_sommerfeld) {
        const BoxSet S = face_slabs(G, box);
        if (S.n > 0)
            BSSN_LAUNCH(KC_SOMMERFELD, k_sommerfeld<R>,
                        dim3(blocks_for(largest(S) * G.ninst), S.n, NCOMP / kSommerfeldGroup),
                        kThreads, stc, u, u64, k, G, S);
    }
    if (with_mom) {
        // The derived fields are differentiated on ext, so they must be valid
        // on ext grown by the first-derivative reach (3); being pointwise, they
        // take the same values there whatever region is computed.
        const Box region = grown_box(box, G, reach + 3);
        BSSN_LAUNCH(KC_MOM_DERIVED, k_mom_derived<R>, blocks_for(box_threads(G, region)), kThreads, stream, u, u64,
                    der, G,
                    region);
    }
    // The FP64 form is bound by FP64 instructions, so its shell slabs avoid
    // divergent closure branches; the FP32 form keeps coalesced slabs.
    const bool coalesced = kPerturbative<R>;
    const SplitBox se = split_box(G, ext, coalesced);
    if (X) {
        cudaEventRecord(X->pre, stream);
        cudaStreamWaitEvent(stb, X->pre, 0);
    }
    // FP32 forms on a grid whose closed axes are Sommerfeld at both ends: one
    // TMA launch over the whole box, closure rows included; else the interior
    // (TMA or generic) and the generic shell slabs beside it.
    bool derivs_whole = false;
    if constexpr (kPerturbative<R>)
        derivs_whole = tma_whole_box(G, box) && launch_first_derivs_tma(u, d1, G, single(ext), with_mom, true, stream);
    if (!derivs_whole) {
        BSSN_LAUNCH_SET(KC_FIRST, 1, (k_first_derivs<R, true>), se.shell, stb, u, der, d1, G, se.shell, with_mom);
        bool derivs_done = false;
        if constexpr (kPerturbative<R>)
            derivs_done = launch_first_derivs_tma(u, d1, G, se.interior, with_mom, false, stream);
        if (!derivs_done)
            BSSN_LAUNCH_SET(KC_FIRST, 0, (k_first_derivs<R, false>), se.interior, stream, u, der, d1, G, se.interior,
                            with_mom);
    }
    if (X) {
        cudaEventRecord(X->fd, stb);
        cudaStreamWaitEvent(stream, X->fd, 0);
    }
    // k_sommerfeld replaces every component's RHS on the active Sommerfeld face
    // planes, so the stencil kernels skip those planes.
    const SplitBox sb = split_box(G, G.any_sommerfeld ? without_faces(G, box) : box, coalesced);
    const R* dmp = with_mom ? static_cast<const R*>(damp) : nullptr;
    if (X) {
        cudaEventRecord(X->d1, stream);
        cudaStreamWaitEvent(stb, X->d1, 0);
        cudaStreamWaitEvent(stc, X->d1, 0);
    }
    // gauge: its own branch (b in the FP64 form, c in the FP32 form)
    const cudaStream_t stg = kPerturbative<R> ? stc : stb;
    // FP32 forms: where every closed axis is closed at both faces, the TMA box
    // kernels apply the closure rows themselves and take the whole box minus
    // the face planes, shell included (tma_whole_box)
    const bool whole = kPerturbative<R> && tma_whole_box(G, box);
    const BoxSet tma_set = whole ? single(without_faces(G, box)) : sb.interior;
    BoxSet none;
    none.n = 0;
    bool gauge_done = false;
    if constexpr (kPerturbative<R>)
        gauge_done = launch_curv_tma(KC_GAUGE, u, u64, d1, nullptr, nullptr, k, G, tma_set, nfield, stg);
    if (!gauge_done)
        BSSN_LAUNCH_SET(KC_GAUGE, 0, (k_rhs_gauge<R, false>), sb.interior, stg, u, u64, d1, k, G, sb.interior,
                        nfield);
    const BoxSet& gauge_shell = gauge_done && whole ? none : sb.shell;
    BSSN_LAUNCH_SET(KC_GAUGE, 1, (k_rhs_gauge<R, true>), gauge_shell, stg, u, u64, d1, k, G, gauge_shell, nfield);
    // the shell's damping and curvature (pointwise in damp) run beside the
    // interior's: on c (FP64) or after the K/Gt RHS on b (FP32)
    const cudaStream_t sts = kPerturbative<R> ? stb : stc;
    if (with_mom) {
        BSSN_LAUNCH_SET(KC_MOM_DAMP, 0, (k_mom_damping<R, false>), sb.interior, stream, u, u64, der, d1, mat, damp, G,
                        sb.interior, nfield);
        BSSN_LAUNCH_SET(KC_MOM_DAMP, 1, (k_mom_damping<R, true>), sb.shell, sts, u, u64, der, d1, mat, damp, G,
                        sb.shell, nfield);
    }
    if constexpr (kPerturbative<R>) {
        // FP32 form: issue- and latency-bound, so the smaller split kernels run
        // at higher occupancy.
        const bool kgt_done = launch_curv_tma(KC_KGT, u, u64, d1, dmp, mat, k, G, tma_set, nfield, stb);
        if (!kgt_done)
            BSSN_LAUNCH_SET(KC_KGT, 0, (k_rhs_kgt<R, false>), sb.interior, stb, u, u64, d1, mat, k, G, sb.interior,
                            nfield);
        const BoxSet& kgt_shell = kgt_done && whole ? none : sb.shell;
        BSSN_LAUNCH_SET(KC_KGT, 1, (k_rhs_kgt<R, true>), kgt_shell, stb, u, u64, d1, mat, k, G, kgt_shell, nfield);
        const bool at_done = launch_curv_tma(KC_AT, u, u64, d1, dmp, mat, k, G, tma_set, nfield, stream);
        if (!at_done)
            BSSN_LAUNCH_SET(KC_AT, 0, (k_rhs_at<R, false>), sb.interior, stream, u, u64, d1, dmp, mat, k, G,
                            sb.interior, nfield);
        const BoxSet& at_shell = at_done && whole ? none : sb.shell;
        BSSN_LAUNCH_SET(KC_AT, 1, (k_rhs_at<R, true>), at_shell, sts, u, u64, d1, dmp, mat, k, G, at_shell, nfield);
    } else {
        BSSN_LAUNCH_SET(KC_CURV, 0, (k_rhs_curv<R, false>), sb.interior, stream, u, u64, d1, dmp, mat, k, G,
                        sb.interior, nfield);
        BSSN_LAUNCH_SET(KC_CURV, 1, (k_rhs_curv<R, true>), sb.shell, sts, u, u64, d1, dmp, mat, k, G, sb.shell,
                        nfield);
    }
    if (X) {
        cudaEventRecord(X->join_b, stb);
        cudaEventRecord(X->join_c, stc);
        cudaStreamWaitEvent(stream, X->join_b, 0);
        cudaStreamWaitEvent(stream, X->join_c, 0);
    }
}

// ---------------------------------------------------------------------------
// The reference's lower triangles of At and gt.  It evolves all nine entries
// of both; the Hessians in W^2 D_i D_j alpha and in the W terms of W^2 R_ij
// are formed as D1_j(D1_i f) for the (i, j) entry (JAX_BSSN/bssn/
// geometry.py:47-56, 131-135), so its lower triangle uses the other ordering
// than its (and this code's) upper triangle.  The two orderings commute in
// exact arithmetic but round differently where the inner derivative's
// one-sided closure acts on O(1) samples, i.e. on the rows next to a
// Sommerfeld face.  The differences dA_ij = At_ji - At_ij and
// dg_ij = gt_ji - gt_ij (i < j) then obey, to first order in them,
//   d_t dA = alpha W (dd_ji W - dd_ij W) - W^2 (dd_ji alpha - dd_ij alpha)
//            + beta.grad dA + KO dA + (alpha K - 2/3 div beta) dA
//            - 1/2 alpha W^2 gt^mn d_m d_n dg,
//   d_t dg = beta.grad dg + KO dg - 2/3 div beta dg - 2 alpha dA,
// dd_ij f = D1_j(D1_i f), and the Sommerfeld condition (zero far value) on the
// active faces (JAX_BSSN/bssn/extrinsic_curvature.py, conformal_metric.py,
// evolution/boundaries.py:20-171, the terms of each that do not cancel
// between (i, j) and (j, i)).  The Ricci term's gt^mn d_m d_n dg matters
// because dg, though of order 1e-17, is as sharp as the closure rows.  Terms
// of second order (At gt^-1 At, the Christoffel terms) are left out.
//
// The differences live on the closure rows (they fall by orders of magnitude
// per row inward), so k_lower_triangle evaluates these rates only on the shell
// slabs of the owned box and the difference fields are zero beyond it.  The
// source -- a difference of two roundings -- is evaluated in FP64 from the
// stored first derivatives as the reference rounds it; the terms linear in
// the differences need only a few digits (they are 1e-17-sized corrections
// of 1e-12-sized values) and run in FP32 on FP32 copies, which keeps the
// shell's stencils off GB300's FP64 pipe.  RK4 stage q reads the stage values
// at the stencil taps from one FP32 buffer (stage 1: the step's values) and
// writes the next stage's values  delta + c dt rate  to the other; stage 4
// adds dt/6 acc to the FP64 delta in place and writes its FP32 copy for the
// next step's stage 1.  Only the reference-layout RK4 call carries the
// differences.
// ---------------------------------------------------------------------------

// D1_n(D1_m f) at ix (m != n): the outer first derivative along n applied to
// the inner one along m at its taps, with the closure rows of both axes.
template <typename R>
__device__ __forceinline__ R mixed_d1(const R* __restrict__ f, const Geo& G, int m, int n, const int (&ix)[3]) {
    const Axis& a = G.ax[n];
    if (a.reduced || G.ax[m].reduced) return R(0);
    const long long s = G.st[n];
    auto inner = [&](int o) { return D1<R, true>(f + o * s, G, m, ix[m]); };
    auto row = [&](const double (&c)[5], int first) {
        R acc = R(0);
#pragma unroll
        for (int t = 0; t < 5; ++t) acc += static_cast<R>(c[t]) * inner(first + t);
        return acc * BSSN_CO(R, G, inv_dx);
    };
    constexpr double L0[5] = {-25.0 / 12.0, 4.0, -3.0, 4.0 / 3.0, -1.0 / 4.0};
    constexpr double L1[5] = {-1.0 / 4.0, -5.0 / 6.0, 3.0 / 2.0, -1.0 / 2.0, 1.0 / 12.0};
    constexpr double R0[5] = {1.0 / 4.0, -4.0 / 3.0, 3.0, -4.0, 25.0 / 12.0};
    constexpr double R1[5] = {-1.0 / 12.0, 1.0 / 2.0, -3.0 / 2.0, 5.0 / 6.0, 1.0 / 4.0};
    int r = right_row<true>(a, ix[n], 2);
    if (r == 0) return row(R0, -4);
    if (r == 1) return row(R1, -3);
    r = left_row<true>(a, ix[n], 2);
    if (r == 0) return row(L0, 0);
    if (r == 1) return row(L1, -1);
    const R c1 = inner(1) - inner(-1), c2 = inner(2) - inner(-2);
    const R d4 = c1 * BSSN_CO(R, G, d1a) + c2 * BSSN_CO(R, G, d1b);
    if (!a.mad) return d4;
    const R c3 = inner(3) - inner(-3);
    return BSSN_AQ(R, a) * d4
           + BSSN_AOMQ(R, a) * ((R(0.75) * c1 - R(0.15) * c2 + c3 / R(60)) * BSSN_CO(R, G, inv_dx));
}

__global__ void __launch_bounds__(kThreads)
k_lower_triangle(const double* __restrict__ u, const double* __restrict__ d1, const float* __restrict__ din,
                 float* __restrict__ dout, double* __restrict__ delta, float* __restrict__ acc, Geo G, BoxSet S,
                 int stage, int nfield) {
    PointCtx c;
    if (!point(S.b[blockIdx.y], c, G)) return;
    const long long cs = G.cs, p = c.p;
    const int k = blockIdx.z;   // pair (0,1), (0,2), (1,2)
    constexpr int pairs[3][2] = {{0, 1}, {0, 2}, {1, 2}};
    const int i = pairs[k][0], j = pairs[k][1];
    const float* fa = din + k * cs + p;          // dA_ij stage values
    const float* fg = din + (3 + k) * cs + p;    // dg_ij stage values
    bool face = false, row1 = false;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        const Axis& a = G.ax[d];
        face = face || (a.slo && c.ix[d] == a.start) || (a.shi && c.ix[d] == a.end - 1);
        row1 = row1 || (a.lbc && c.ix[d] == a.start + 1) || (a.rbc && c.ix[d] == a.end - 2);
    }
    float ra, rg;
    if (face) {
        float X[3];
#pragma unroll
        for (int d = 0; d < 3; ++d) X[d] = (float)(G.ax[d].xmin + G.dx * (double)(c.ix[d] - G.ax[d].org));
        const float r = sqrtf(X[0] * X[0] + X[1] * X[1] + X[2] * X[2]);
        const float rs = r > 0.0f ? r : 1.0f;
        float radial_a = 0.0f, radial_g = 0.0f;
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            radial_a += X[d] * D1<float, true>(fa, G, d, c.ix[d]);
            radial_g += X[d] * D1<float, true>(fg, G, d, c.ix[d]);
        }
        ra = -(radial_a + fa[0]) / rs;
        rg = -(radial_g + fg[0]) / rs;
    } else {
        const double W = u[CW * cs + p], al = u[CALPHA * cs + p];
        // the commuted Hessians' difference (the source), as the reference
        // rounds it: on the second row from a face, where the inner
        // derivative's one-sided closure acts (further in, both orderings use
        // centred stencils and the difference is below 1e-20)
        float src = 0.0f;
        if (row1) {
            const double wu = D1<double, true>(d1ptr(d1, G, nfield, i, MIX_W, p), G, j, c.ix[j]);
            const double wl = D1<double, true>(d1ptr(d1, G, nfield, j, MIX_W, p), G, i, c.ix[i]);
            const double au = D1<double, true>(d1ptr(d1, G, nfield, i, MIX_ALPHA, p), G, j, c.ix[j]);
            const double al_ = D1<double, true>(d1ptr(d1, G, nfield, j, MIX_ALPHA, p), G, i, c.ix[i]);
            src = (float)(al * W * (wl - wu) - W * W * (al_ - au));
        }
        float beta[3], bs[3], g[6], gi[6];
#pragma unroll
        for (int s6 = 0; s6 < 6; ++s6) g[s6] = (float)u[(GXX + s6) * cs + p];
        inverse_metric(g, gi);
        float divb = 0.0f;
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            beta[d] = (float)u[(BX + d) * cs + p];
            divb += (float)d1ptr(d1, G, nfield, d, MIX_B + d, p)[0];
        }
        shift_over_12dx(G, beta, bs);
        const float fal = (float)al, fW = (float)W, fK = (float)u[CK * cs + p];
        // gt^mn d_m d_n dg
        float lap = 0.0f;
#pragma unroll
        for (int m = 0; m < 3; ++m) {
            lap += gi[sym(m, m)] * D2<float, true, false>(fg, G, m, c.ix[m]);
#pragma unroll
            for (int n = m + 1; n < 3; ++n) lap += 2.0f * gi[sym(m, n)] * mixed_d1(fg, G, m, n, c.ix);
        }
        const float da = fa[0], dg = fg[0];
        ra = src + ADV<float, true, false>(fa, G, c.ix, beta, bs) + KO<float, true, false>(fa, G, c.ix)
             + (fal * fK - (2.0f / 3.0f) * divb) * da - 0.5f * fal * fW * fW * lap;
        rg = ADV<float, true, false>(fg, G, c.ix, beta, bs) + KO<float, true, false>(fg, G, c.ix)
             - (2.0f / 3.0f) * divb * dg - 2.0f * fal * da;
    }
    const long long qa = k * cs + p, qg = (3 + k) * cs + p;
    float aa = ra, ag = rg;
    if (stage > 1) {
        const float w = stage == 4 ? 1.0f : 2.0f;
        aa = fmaf(w, ra, acc[qa]);
        ag = fmaf(w, rg, acc[qg]);
    }
    if (stage < 4) {
        acc[qa] = aa;
        acc[qg] = ag;
        const double h = stage == 3 ? G.dt : 0.5 * G.dt;
        dout[qa] = (float)fma(h, (double)ra, delta[qa]);
        dout[qg] = (float)fma(h, (double)rg, delta[qg]);
    } else {
        const double na = fma(G.dt / 6.0, (double)aa, delta[qa]);
        const double ng = fma(G.dt / 6.0, (double)ag, delta[qg]);
        delta[qa] = na;
        delta[qg] = ng;
        dout[qa] = (float)na;   // the next step's stage-1 values
        dout[qg] = (float)ng;
    }
}

cudaError_t launch_lower_triangle(const double* u, const RhsWork& w, const LowerTriangle& lt, const Geo& G,
                                  const Box& box, int stage, cudaStream_t stream) {
    const int nfield = G.kappa != 0.0 ? NMIX + NMIX_MOM : NMIX;
    const BoxSet shell = split_box(G, box, false).shell;
    if (shell.n == 0) return cudaSuccess;
    const int threads = set_threads(shell, 1);
    const dim3 grid((unsigned)((largest(shell) + threads - 1) / threads), shell.n, 3);
    BSSN_LAUNCH(KC_OTHER, k_lower_triangle, grid, threads, stream, u, w.d1, lower_triangle_input(lt, stage),
                lower_triangle_output(lt, stage), lt.delta, lt.acc, G, shell, stage, nfield);
    return cudaGetLastError();
}

cudaError_t launch_inner_derivs(const double* u, double* d1, const Geo& G, const Box& box, cudaStream_t stream) {
    // periodic boxes have no closure rows: the closure-free instantiation
    // covers the box grown by the composition reach; with Sommerfeld faces
    // the closure rows take the general one (closed axes are not grown)
    const BoxSet es = single(grown_box(box, G, composition_reach(G)));
    if (G.any_sommerfeld)
        BSSN_LAUNCH_SET(KC_FIRST, 1, (k_first_derivs<double, true>), es, stream, u, (const double*)nullptr, d1, G, es,
                        0);
    else
        BSSN_LAUNCH_SET(KC_FIRST, 0, (k_first_derivs<double, false>), es, stream, u, (const double*)nullptr, d1, G, es,
                        0);
    return cudaGetLastError();
}

cudaError_t tune_rhs(const double* u, double* k, const RhsWork& w, const Geo& G, const Box& box, cudaStream_t s,
                     int reps, float margin, std::string* report) {
    cudaStreamCaptureStatus status = cudaStreamCaptureStatusNone;
    cudaError_t e = cudaStreamIsCapturing(s, &status);
    if (e != cudaSuccess) return e;
    if (status != cudaStreamCaptureStatusNone) return cudaErrorStreamCaptureUnsupported;
    int dev = 0;
    if ((e = cudaGetDevice(&dev)) != cudaSuccess) return e;
    std::vector<int> classes = {KC_FIRST, KC_GAUGE};
    if (float_form(G.precision)) {
        classes.push_back(KC_KGT);
        classes.push_back(KC_AT);
    } else {
        classes.push_back(KC_CURV);
    }
    if (G.kappa != 0.0) classes.push_back(KC_MOM_DAMP);
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if ((e = cudaEventCreate(&e0)) != cudaSuccess) return e;
    if ((e = cudaEventCreate(&e1)) != cudaSuccess) {
        cudaEventDestroy(e0);
        return e;
    }
    auto time_rhs = [&](float& ms) -> cudaError_t {
        cudaError_t r = cudaEventRecord(e0, s);
        for (int i = 0; i < reps && r == cudaSuccess; ++i) r = launch_rhs(u, k, w, G, box, s);
        if (r == cudaSuccess) r = cudaEventRecord(e1, s);
        if (r == cudaSuccess) r = cudaEventSynchronize(e1);
        if (r == cudaSuccess) r = cudaEventElapsedTime(&ms, e0, e1);
        return r;
    };
    float ms = 0.0f, base = 0.0f;
    e = time_rhs(ms);   // warm-up (streams, caches)
    // the current shapes' time: a candidate must come in under margin x it
    if (e == cudaSuccess) e = time_rhs(base);
    for (size_t c = 0; c < classes.size() && e == cudaSuccess; ++c) {
        for (int shell = 0; shell < 2 && e == cudaSuccess; ++shell) {
            int best = 0;
            float best_ms = 0.0f;
            long long size = -1;
            for (int t : kTuneCandidates) {
                t_force_cls = classes[c];
                t_force_shell = shell;
                t_force_threads = t;
                t_seen_size = -1;
                e = time_rhs(ms);
                if (e != cudaSuccess || t_seen_size < 0) break;   // slot not launched here
                size = t_seen_size;
                if (best == 0 || ms < best_ms) {
                    best = t;
                    best_ms = ms;
                }
            }
            t_force_cls = t_force_shell = -1;
            if (e != cudaSuccess || size < 0 || best == 0) continue;
            if (best_ms > margin * base) {
                if (report)
                    *report += "class " + std::to_string(classes[c]) + (shell ? " shell" : " interior") +
                               ": heuristic kept; ";
                continue;
            }
            {
                std::lock_guard<std::mutex> guard(g_tune_lock);
                g_tuned[TuneKey{dev, classes[c], shell, G.precision, size}] = best;
            }
            base = best_ms;   // later slots are measured against the tuned whole
            if (report)
                *report += "class " + std::to_string(classes[c]) + (shell ? " shell" : " interior") + ": " +
                           std::to_string(best) + " threads (" + std::to_string(best_ms / reps) + " ms per RHS); ";
        }
    }
    t_force_cls = t_force_shell = -1;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return e;
}

cudaError_t launch_rhs_f32_prepared(const double* u, double* k, const RhsWork& w, const Geo& G, const Box& box,
                                    cudaStream_t stream) {
    launch_rhs_form<float>(w.uf, u, k, w.d1f, w.derf, w.dampf, w.mat, G, box, stream);
    return cudaGetLastError();
}

cudaError_t launch_rhs(const double* u, double* k, const RhsWork& w, const Geo& G, const Box& box,
                       cudaStream_t stream) {
    if (float_form(G.precision)) {
        // Every sample the RHS kernels read lies within 6 of the box: first
        // derivatives on the box grown by 3 with a 3-sample reach; KO and
        // upwind stencils reach 4.
        const Box region = grown_box(box, G, 6);
        // background: each component's value at the box's first sample
        const long long p0 = (long long)box.lo[0] * G.st[0] + (long long)box.lo[1] * G.st[1] + box.lo[2];
        BSSN_LAUNCH(KC_CONVERT, k_perturb, blocks_for(box_threads(G, region)), kThreads, stream, u, w.uf, G, region,
                    p0);
        launch_rhs_form<float>(w.uf, u, k, w.d1f, w.derf, w.dampf, w.mat, G, box, stream);
    } else {
        launch_rhs_form<double>(u, u, k, w.d1, w.der, w.damp, w.mat, G, box, stream);
    }
    return cudaGetLastError();
}

}  // namespace bssn
