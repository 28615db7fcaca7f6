// Reverse-mode (adjoint) kernels of the BSSN evolution on GB300.
//
// The forward path is rk4_step (JAX_BSSN/evolution/time_evolve.py:144-217)
// with its RHS compute_bssn_rhs (time_evolve.py:41-57).  The reference never
// differentiates it; jax.grad through it would be XLA's reverse mode.  Here
// the vector-Jacobian products are written as kernels:
//
//   RHS.  At every point the RHS is F(x) + advection + dissipation, where x
//   holds the 21 state values and their first and second finite-difference
//   derivatives (132 inputs) and F is algebraic.  For an adjoint kbar of the
//   RHS:
//     k_adj_point   recomputes x from the state (the forward's own stencil
//                   helpers), runs the generated reverse sweep of F
//                   (bssn_adjoint_point.cuh) and writes the 21 value
//                   coefficients into the state adjoint and the 111
//                   derivative coefficients into their own blocks;
//     k_adj_mixed   folds each composed mixed derivative D1_n(D1_m f) (m < n)
//                   into the first-derivative coefficient of axis m:
//                   on a periodic grid the centred D1 is antisymmetric
//                   (D1^T = -D1) and D2 and the sixth difference symmetric,
//                   so  m_a = -c1_a + sum_{b>a} D1_b(c2_ab);
//     k_adj_field   applies the transposed stencils: sum_a D1_a(m_a) +
//                   D2_a(c2_aa), the (symmetric) Kreiss-Oliger term of kbar,
//                   and the transposed upwind advection -- at each neighbour
//                   the stencil side is the one the sign of that neighbour's
//                   shift selected in the forward -- plus the shift's own
//                   adjoint from the advection terms, sum_f kbar_f U_a(f).
//   Projection and stage combination.  k_adj_final, k_adj_stage and
//   k_adj_initial run the generated reverse sweep of the algebraic projection
//   (time_evolve.py:94-141) on the pre-projection values and distribute the
//   result over the RK4 combination's inputs.
//
// Evolutions are differentiated with sqrt(N) checkpointing: the forward pass
// stores the state every `segment` steps; the backward pass re-runs each
// segment from its checkpoint, keeping the step-start states and, by
// store_stages: 0 nothing more (each step's stages are recomputed once more),
// 1 every step's four stage RHS values (the stage states are then re-formed by
// the cheap stage kernels), 2 the stage states as well.  With 1 or 2 the
// forward pass records the last segment itself.
// Everything runs on instance batches (layout [component][instance][block]).
// Scope: each axis periodic or closed by Sommerfeld faces at both ends (the
// band kernels below); kappa = 0, no matter, FP64 arithmetic.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>

#include "../../include/bssn_gb300.h"
#include "bssn_adjoint_point.cuh"
#include "bssn_driver.h"
#include "bssn_profile.h"

namespace bssn {
namespace adjoint {
namespace {

constexpr int kThreads = 128;
constexpr int NC1 = 45;            // first-derivative coefficient blocks
constexpr int NC2 = 66;            // second-derivative coefficient blocks
constexpr int NCOEF = NC1 + NC2;   // 111
constexpr int I_DG = 21, I_DW = 39, I_DAL = 42, I_DK = 45, I_DB = 48, I_DGT = 57;
constexpr int I_D2G = 66, I_D2W = 102, I_D2AL = 108, I_D2B = 114;

inline unsigned blocks_of(long long n) { return (unsigned)((n + kThreads - 1) / kThreads); }

// Coefficient block (index into the 111) of d_a of state component f, or -1.
__host__ __device__ constexpr int c1_block(int f, int a) {
    return f < 6 ? I_DG - 21 + 6 * a + f
         : f == CW ? I_DW - 21 + a
         : f == CK ? I_DK - 21 + a
         : (f >= GTX && f <= GTZ) ? I_DGT - 21 + 3 * a + (f - GTX)
         : f == CALPHA ? I_DAL - 21 + a
         : (f >= BX) ? I_DB - 21 + 3 * (f - BX) + a
         : -1;
}

// Coefficient block of d_m d_n of the NMIX field mf (pair slot pr), f's slot
// in the 111.
__host__ __device__ constexpr int c2_block(int mf, int pr) {
    return mf < 6 ? I_D2G - 21 + 6 * pr + mf
         : mf == MIX_W ? I_D2W - 21 + pr
         : mf == MIX_ALPHA ? I_D2AL - 21 + pr
         : I_D2B - 21 + 6 * (mf - MIX_B) + pr;
}

// NMIX field index of state component f (gt, W, alpha, beta), or -1.
__host__ __device__ constexpr int mix_of(int f) {
    return f < 6 ? f : f == CW ? MIX_W : f == CALPHA ? MIX_ALPHA : (f >= BX ? MIX_B + (f - BX) : -1);
}

PointParams point_params(const Geo& G) {
    PointParams pp;
    pp.eta = G.eta;
    pp.gdrv = G.g;
    pp.c_harm = G.gauge == 0 ? 1.0 : 0.0;
    pp.c_log = G.gauge == 1 ? 1.0 : 0.0;
    pp.shift_on = G.zero_shift ? 0.0 : 1.0;
    return pp;
}

struct Pt {
    int ix[3];
    long long p;
};

__device__ __forceinline__ bool owned_point(const Geo& G, const Box& B, Pt& c) {
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= box_threads(G, B)) return false;
    const long long off = instance_offset(G, B, t);
    B.coords(t, c.ix);
    c.p = lin(G, c.ix) + off;
    return true;
}

// ---------------------------------------------------------------------------
// Sommerfeld faces.  On an axis closed by Sommerfeld faces the forward
// replaces the RHS on the face planes by the radial condition and uses
// one-sided rows next to them: D1 and D2 on rows 0-1 from a face, the sixth
// difference on rows 0-2, and the centred D1 in place of the upwind one for
// advection on rows 0-2 (JAX_BSSN/evolution/derivatives.py:42-338,
// spatial_derivatives.py:18-92, boundaries.py:150-171).  Rows 0-2 at each
// closed face form the axis' band.  The interior transposes gather from the
// sources outside the bands (masked taps); sources in a band scatter their
// rows' own weights with atomic adds (k_adj_band_mixed, k_adj_band_field).
// The face planes' bulk RHS is never formed, so their kbar enters only the
// transpose of the radial condition (k_adj_sommerfeld).
// ---------------------------------------------------------------------------
struct BandRow {
    int r;        // row from the nearer closed face (0..2), or -1
    bool right;   // that face is the upper one
};
// The upper face is checked first, as the forward's closures do.
__device__ __forceinline__ BandRow band_row(const Axis& A, int i) {
    if (A.rbc) {
        const int r = A.end - 1 - i;
        if (r >= 0 && r < 3) return {r, true};
    }
    if (A.lbc) {
        const int r = i - A.start;
        if (r >= 0 && r < 3) return {r, false};
    }
    return {-1, false};
}
// Sources the interior transposes gather along A: outside the bands and not
// beyond a closed face.
__device__ __forceinline__ bool gathers(const Axis& A, int i) {
    return !(A.lbc && i < A.start + 3) && !(A.rbc && i > A.end - 4);
}
__device__ __forceinline__ bool face_along(const Axis& A, int i) {
    return (A.slo && i == A.start) || (A.shi && i == A.end - 1);
}
// A point whose RHS the forward replaces by the radial condition.
__device__ __forceinline__ bool face_point(const Geo& G, const int (&ix)[3]) {
    return face_along(G.ax[0], ix[0]) || face_along(G.ax[1], ix[1]) || face_along(G.ax[2], ix[2]);
}
// ... on a face plane of an axis other than a: then so is every source
// along a of this point.
__device__ __forceinline__ bool face_off_axis(const Geo& G, const int (&ix)[3], int a) {
    bool f = false;
#pragma unroll
    for (int d = 0; d < 3; ++d) f = f || (d != a && face_along(G.ax[d], ix[d]));
    return f;
}

// One-sided rows at the lower face (row r's taps start at offset -r); the
// upper face's are their mirror images (odd in the offset for D1).
__constant__ double kBandD1[2][5] = {{-25.0 / 12.0, 4.0, -3.0, 4.0 / 3.0, -1.0 / 4.0},
                                      {-1.0 / 4.0, -5.0 / 6.0, 3.0 / 2.0, -1.0 / 2.0, 1.0 / 12.0}};
__constant__ double kBandD2[2][6] = {{15.0 / 4.0, -77.0 / 6.0, 107.0 / 6.0, -13.0, 61.0 / 12.0, -5.0 / 6.0},
                                      {5.0 / 6.0, -5.0 / 4.0, -1.0 / 3.0, 7.0 / 6.0, -1.0 / 2.0, 1.0 / 12.0}};
__constant__ double kBandKO[3][8] = {{4.0, -27.0, 78.0, -125.0, 120.0, -69.0, 22.0, -3.0},
                                      {3.0, -20.0, 57.0, -90.0, 85.0, -48.0, 15.0, -2.0},
                                      {2.0, -13.0, 36.0, -55.0, 50.0, -27.0, 8.0, -1.0}};
// centred rows, offsets -2..2
__constant__ double kMidD1[5] = {1.0 / 12.0, -2.0 / 3.0, 0.0, 2.0 / 3.0, -1.0 / 12.0};
__constant__ double kMidD2[5] = {-1.0 / 12.0, 16.0 / 12.0, -30.0 / 12.0, 16.0 / 12.0, -1.0 / 12.0};
__constant__ double kMidKO[7] = {1.0, -6.0, 15.0, -20.0, 15.0, -6.0, 1.0};

enum BandOp { kOpD1 = 0, kOpD2 = 1, kOpKO = 2 };
// Calls tap(offset, weight) for every tap of the row the forward applies at
// band row b (b.r < 0: an interior sample), weights before the operator's
// factor (1/dx, 1/dx^2, the KO factor).  D1 and D2 are one-sided on rows 0-1
// and centred beyond; the sixth difference is one-sided on rows 0-2.
template <typename F>
__device__ __forceinline__ void band_taps(int op, BandRow b, F&& tap) {
    if (op == kOpKO && b.r >= 0) {
#pragma unroll
        for (int t = 0; t < 8; ++t) {
            const int o = t - b.r;
            tap(b.right ? -o : o, kBandKO[b.r][t]);
        }
    } else if (op == kOpKO) {
#pragma unroll
        for (int t = 0; t < 7; ++t) tap(t - 3, kMidKO[t]);
    } else if (b.r < 0 || b.r > 1) {
#pragma unroll
        for (int t = 0; t < 5; ++t) tap(t - 2, op == kOpD1 ? kMidD1[t] : kMidD2[t]);
    } else if (op == kOpD1) {
#pragma unroll
        for (int t = 0; t < 5; ++t) {
            const int o = t - b.r;
            tap(b.right ? -o : o, b.right ? -kBandD1[b.r][t] : kBandD1[b.r][t]);
        }
    } else {
#pragma unroll
        for (int t = 0; t < 6; ++t) {
            const int o = t - b.r;
            tap(b.right ? -o : o, kBandD2[b.r][t]);
        }
    }
}

// The forward's centred D1 and D2 along axis a at index j of x (x points at
// sample j) over the sources the gathers take; on periodic geometries the
// forward's own stencil (every source, MAD blend included).
template <bool Closed>
__device__ __forceinline__ double g_d1(const double* x, const Geo& G, int a, int j) {
    if constexpr (!Closed) {
        return D1<double, false>(x, G, a, j);
    } else {
        const Axis& A = G.ax[a];
        const long long s = G.st[a];
        auto v = [&](int o) { return gathers(A, j + o) ? x[o * s] : 0.0; };
        return (v(1) - v(-1)) * G.d1a + (v(2) - v(-2)) * G.d1b;
    }
}
template <bool Closed>
__device__ __forceinline__ double g_d2(const double* x, const Geo& G, int a, int j) {
    if constexpr (!Closed) {
        return D2<double, false, false>(x, G, a, j);
    } else {
        const Axis& A = G.ax[a];
        const long long s = G.st[a];
        auto v = [&](int o) { return gathers(A, j + o) ? x[o * s] : 0.0; };
        return ((16.0 * (v(1) + v(-1)) - (v(2) + v(-2))) + -30.0 * v(0)) * G.inv_12dx2;
    }
}

// ---------------------------------------------------------------------------
// point kernel: inputs of F by the forward's stencil helpers, reverse sweep
// ---------------------------------------------------------------------------
template <bool Closed>
__global__ void __launch_bounds__(kThreads)
k_adj_point(const double* __restrict__ u, const double* __restrict__ d1, const double* __restrict__ kbar,
            double kscale, double* __restrict__ ubar, double* __restrict__ coef, Geo G, Box B, PointParams pp,
            int accumulate) {
    Pt c;
    if (!owned_point(G, B, c)) return;
    const long long cs = G.cs, p = c.p;
    if constexpr (Closed) {
        if (face_point(G, c.ix)) {   // the forward replaces this RHS: no bulk terms
            if (!accumulate)
                for (int f = 0; f < NCOMP; ++f) ubar[f * cs + p] = 0.0;
            for (int k = 0; k < NCOEF; ++k) coef[(long long)k * cs + p] = 0.0;
            return;
        }
    }
    double x[kPointInputs];
#pragma unroll
    for (int f = 0; f < NCOMP; ++f) x[f] = u[f * cs + p];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
#pragma unroll
        for (int s = 0; s < 6; ++s) x[I_DG + 6 * a + s] = D1<double, Closed>(u + (GXX + s) * cs + p, G, a, c.ix[a]);
        x[I_DW + a] = D1<double, Closed>(u + CW * cs + p, G, a, c.ix[a]);
        x[I_DAL + a] = D1<double, Closed>(u + CALPHA * cs + p, G, a, c.ix[a]);
        x[I_DK + a] = D1<double, Closed>(u + CK * cs + p, G, a, c.ix[a]);
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            x[I_DB + 3 * i + a] = D1<double, Closed>(u + (BX + i) * cs + p, G, a, c.ix[a]);
            x[I_DGT + 3 * a + i] = D1<double, Closed>(u + (GTX + i) * cs + p, G, a, c.ix[a]);
        }
    }
    // second derivatives: D2 on the diagonal, D1 along the larger axis of the
    // stored first derivative along the smaller one off it (the forward's order)
#pragma unroll
    for (int m = 0; m < 3; ++m)
#pragma unroll
        for (int n = m; n < 3; ++n) {
            const int pr = sym(m, n);
#pragma unroll
            for (int f = 0; f < NMIX; ++f) {
                const double v = m == n
                    ? D2<double, Closed, false>(u + mix_source(f) * cs + p, G, m, c.ix[m])
                    : D1<double, Closed>(d1 + (long long)(m * NMIX + f) * cs + p, G, n, c.ix[n]);
                x[21 + c2_block(f, pr)] = v;
            }
        }
    double kb[NCOMP];
#pragma unroll
    for (int f = 0; f < NCOMP; ++f) kb[f] = kscale * kbar[f * cs + p];
    double xb[kPointInputs];
    rhs_point_vjp(x, kb, pp, xb);
#pragma unroll
    for (int f = 0; f < NCOMP; ++f) ubar[f * cs + p] = accumulate ? ubar[f * cs + p] + xb[f] : xb[f];
#pragma unroll
    for (int k = 0; k < NCOEF; ++k) coef[(long long)k * cs + p] = xb[21 + k];
}

// m_a = -c1_a + sum_{b > a} D1_b(c2_ab) for the NMIX fields, into mbuf
// (layout of the inner-derivative buffer: block a * NMIX + f).
template <bool Closed>
__global__ void __launch_bounds__(kThreads)
k_adj_mixed(const double* __restrict__ coef, double* __restrict__ mbuf, Geo G, Box B) {
    Pt c;
    if (!owned_point(G, B, c)) return;
    const long long cs = G.cs, p = c.p;
#pragma unroll 1
    for (int f = 0; f < NMIX; ++f) {
        const int comp = mix_source(f);
        const double* c01 = coef + (long long)c2_block(f, sym(0, 1)) * cs + p;
        const double* c02 = coef + (long long)c2_block(f, sym(0, 2)) * cs + p;
        const double* c12 = coef + (long long)c2_block(f, sym(1, 2)) * cs + p;
        const double m0 = -coef[(long long)c1_block(comp, 0) * cs + p] + g_d1<Closed>(c01, G, 1, c.ix[1])
                          + g_d1<Closed>(c02, G, 2, c.ix[2]);
        const double m1 = -coef[(long long)c1_block(comp, 1) * cs + p] + g_d1<Closed>(c12, G, 2, c.ix[2]);
        const double m2 = -coef[(long long)c1_block(comp, 2) * cs + p];
        mbuf[(long long)(0 * NMIX + f) * cs + p] = m0;
        mbuf[(long long)(1 * NMIX + f) * cs + p] = m1;
        mbuf[(long long)(2 * NMIX + f) * cs + p] = m2;
    }
}

// Upwind weights of offset k (index k + 4, k in [-4, 4]) for a positive and a
// negative coefficient: D4 in units of 1/(12 dx), the sixth-order side
// stencils in units of 1/(60 dx) (JAX_BSSN/evolution/derivatives.py:166-338).
__constant__ double kUp4[2][9] = {{0, 0, 0, -3, -10, 18, -6, 1, 0}, {0, -1, 6, -18, 10, 3, 0, 0, 0}};
__constant__ double kUp6[2][9] = {{0, 0, 2, -24, -35, 80, -30, 8, -1}, {1, -8, 30, -80, 35, 24, -2, 0, 0}};

// Transposed stencils of every component at one point, the dissipation and
// advection transposes, and the shift's adjoint from the advection terms
// (with Sommerfeld faces: the gathered part; k_adj_band_field adds the band
// sources').
template <bool Closed>
__global__ void __launch_bounds__(kThreads)
k_adj_field(const double* __restrict__ u, const double* __restrict__ kbar, double kscale,
            const double* __restrict__ coef, const double* __restrict__ mbuf, double* __restrict__ ubar, Geo G,
            Box B) {
    Pt c;
    if (!owned_point(G, B, c)) return;
    const long long cs = G.cs, p = c.p;
    // bulk[a]: the sources along a carry a bulk RHS (not on another axis' face plane)
    bool bulk[3] = {true, true, true};
    if constexpr (Closed) {
#pragma unroll
        for (int a = 0; a < 3; ++a) bulk[a] = !face_off_axis(G, c.ix, a);
    }
    // w[a][k + 4]: weight of kbar_f at q - k e_a in the transposed advection
    double w[3][9];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const Axis& ax = G.ax[a];
        const long long s = G.st[a];
#pragma unroll
        for (int k = -4; k <= 4; ++k) {
            bool take = !ax.reduced;
            if constexpr (Closed) take = take && bulk[a] && gathers(ax, c.ix[a] - k);
            const double b = take ? u[(BX + a) * cs + p - k * s] : 0.0;
            const int side = b > 0.0 ? 0 : 1;
            double c4 = kUp4[side][k + 4] * G.inv_12dx;
            if (ax.mad) c4 = ax.q * c4 + ax.omq * (kUp6[side][k + 4] * G.inv_60dx);
            w[a][k + 4] = b == 0.0 ? 0.0 : b * c4;
        }
    }
    // Where the shift vanishes on every tap of every lane of the warp the
    // transposed advection is exactly zero: skip its taps (warp-uniform).
    bool moving = false;
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int k = 0; k < 9; ++k) moving = moving || w[a][k] != 0.0;
    moving = __any_sync(__activemask(), moving);
    double shift_bar[3] = {0.0, 0.0, 0.0};
    double beta[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) beta[a] = u[(BX + a) * cs + p];
#pragma unroll 1
    for (int f = 0; f < NCOMP; ++f) {
        double r = ubar[f * cs + p];
        const int mf = mix_of(f);
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            if (mf >= 0) {
                r += g_d1<Closed>(mbuf + (long long)(a * NMIX + mf) * cs + p, G, a, c.ix[a]);
                r += g_d2<Closed>(coef + (long long)c2_block(mf, sym(a, a)) * cs + p, G, a, c.ix[a]);
            } else {
                const int cb = c1_block(f, a);
                if (cb >= 0) r -= g_d1<Closed>(coef + (long long)cb * cs + p, G, a, c.ix[a]);
            }
        }
        const bool row_on = !(f >= BX && G.zero_shift);
        if (row_on) {
            const double* kf = kbar + f * cs + p;
            double lin;
            if constexpr (Closed) {
                double t = 0.0;
#pragma unroll
                for (int a = 0; a < 3; ++a) {
                    if (!bulk[a]) continue;
                    const Axis& A = G.ax[a];
                    const long long s = G.st[a];
#pragma unroll
                    for (int o = -3; o <= 3; ++o)
                        if (gathers(A, c.ix[a] + o)) t = fma(kMidKO[o + 3], kf[o * s], t);
                }
                lin = G.ko_scale * t;
            } else {
                lin = KO<double, false, false>(kf, G, c.ix);
            }
            if (moving) {
                double adv = 0.0;
#pragma unroll
                for (int a = 0; a < 3; ++a) {
                    const long long s = G.st[a];
#pragma unroll
                    for (int k = -4; k <= 4; ++k) adv = fma(w[a][k + 4], kf[-k * s], adv);
                }
                lin += adv;
            }
            r = fma(kscale, lin, r);
            // the shift's adjoint from this point's own advection terms (none
            // on a face plane, whose RHS the radial condition replaces)
            bool own = true;
            if constexpr (Closed) own = !face_point(G, c.ix);
            if (own) {
                const double kq = kscale * kf[0];
#pragma unroll
                for (int a = 0; a < 3; ++a)
                    shift_bar[a] =
                        fma(kq, UP1<double, Closed, false>(u + f * cs + p, G, a, c.ix[a], beta[a]), shift_bar[a]);
            }
        }
        ubar[f * cs + p] = r;
    }
#pragma unroll
    for (int a = 0; a < 3; ++a) ubar[(BX + a) * cs + p] += shift_bar[a];
}

// Band sources of the mixed-derivative transposes: mbuf_a(f) -= D1_b^T of the
// c2_ab coefficients at sources in axis b's band (the old sign convention of
// k_adj_mixed: mbuf holds -(c1_a + sum_b D1_b^T c2_ab)).
__global__ void __launch_bounds__(kThreads)
k_adj_band_mixed(const double* __restrict__ coef, double* __restrict__ mbuf, Geo G, Box B) {
    Pt c;
    if (!owned_point(G, B, c)) return;
    const long long cs = G.cs, p = c.p;
#pragma unroll 1
    for (int b = 1; b < 3; ++b) {
        const BandRow br = band_row(G.ax[b], c.ix[b]);
        if (br.r < 0) continue;
        const long long s = G.st[b];
#pragma unroll 1
        for (int f = 0; f < NMIX; ++f)
#pragma unroll 1
            for (int a = 0; a < b; ++a) {
                const double v = coef[(long long)c2_block(f, sym(a, b)) * cs + p] * G.inv_dx;
                if (v == 0.0) continue;
                double* dst = mbuf + (long long)(a * NMIX + f) * cs + p;
                band_taps(kOpD1, br, [&](int o, double wt) { atomicAdd(dst + o * s, -wt * v); });
            }
    }
}

// Band sources of the field transposes: for each closed axis a whose band
// holds this point, the first- and second-derivative transposes of its
// coefficients and, off the face planes, the dissipation and advection
// transposes of its kbar, each with the row's own weights.
__global__ void __launch_bounds__(kThreads)
k_adj_band_field(const double* __restrict__ u, const double* __restrict__ kbar, double kscale,
                 const double* __restrict__ coef, const double* __restrict__ mbuf, double* __restrict__ ubar, Geo G,
                 Box B) {
    Pt c;
    if (!owned_point(G, B, c)) return;
    const long long cs = G.cs, p = c.p;
    const bool face = face_point(G, c.ix);
#pragma unroll 1
    for (int a = 0; a < 3; ++a) {
        const BandRow br = band_row(G.ax[a], c.ix[a]);
        if (br.r < 0) continue;
        const long long s = G.st[a];
        const double beta = u[(BX + a) * cs + p];
#pragma unroll 1
        for (int f = 0; f < NCOMP; ++f) {
            double* dst = ubar + f * cs + p;
            const int mf = mix_of(f);
            double v1, v2 = 0.0;   // D1 and D2 transposes' source values (times their factors)
            if (mf >= 0) {
                v1 = -mbuf[(long long)(a * NMIX + mf) * cs + p] * G.inv_dx;
                v2 = coef[(long long)c2_block(mf, sym(a, a)) * cs + p] * G.inv_dx2;
            } else {
                const int cb = c1_block(f, a);
                v1 = cb >= 0 ? coef[(long long)cb * cs + p] * G.inv_dx : 0.0;
            }
            double vko = 0.0;
            if (!face && !(f >= BX && G.zero_shift)) {
                const double kb = kscale * kbar[f * cs + p];
                v1 += beta * kb * G.inv_dx;   // advection: the centred D1 rows
                vko = kb * G.ko_scale;
            }
            if (v1 != 0.0) band_taps(kOpD1, br, [&](int o, double wt) { atomicAdd(dst + o * s, wt * v1); });
            if (v2 != 0.0) band_taps(kOpD2, br, [&](int o, double wt) { atomicAdd(dst + o * s, wt * v2); });
            if (vko != 0.0) band_taps(kOpKO, br, [&](int o, double wt) { atomicAdd(dst + o * s, wt * vko); });
        }
    }
}

// Transpose of the radial condition on the face planes
// (JAX_BSSN/evolution/boundaries.py:150-171): k_f = -(x^d D1_d f + f - f_far) / r
// scatters -kbar_f / r to the point and -kbar_f x^d / r through each axis' D1
// row.
__global__ void __launch_bounds__(kThreads)
k_adj_sommerfeld(const double* __restrict__ kbar, double kscale, double* __restrict__ ubar, Geo G, Box B) {
    Pt c;
    if (!owned_point(G, B, c)) return;
    if (!face_point(G, c.ix)) return;
    const long long cs = G.cs, p = c.p;
    double X[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) X[d] = G.ax[d].xmin + G.dx * (double)(c.ix[d] - G.ax[d].org);
    const double r = sqrt(X[0] * X[0] + X[1] * X[1] + X[2] * X[2]);
    const double rs = r > 0.0 ? r : 1.0;
#pragma unroll 1
    for (int f = 0; f < NCOMP; ++f) {
        const double kb = kscale * kbar[f * cs + p];
        if (kb == 0.0) continue;
        double* dst = ubar + f * cs + p;
        atomicAdd(dst, -kb / rs);
#pragma unroll 1
        for (int d = 0; d < 3; ++d) {
            const double g = -kb * X[d] / rs * G.inv_dx;
            const Axis& A = G.ax[d];
            const BandRow br = band_row(A, c.ix[d]);
            const long long s = G.st[d];
            const int L = A.end - A.start;
            // along a periodic axis a tap beyond the owned samples is the
            // ghost copy of an owned one: its adjoint goes to that sample
            band_taps(kOpD1, br, [&](int o, double wt) {
                int i = c.ix[d] + o;
                if (!A.lbc && !A.rbc) i = i < A.start ? i + L : (i >= A.end ? i - L : i);
                atomicAdd(dst + (long long)(i - c.ix[d]) * s, wt * g);
            });
        }
    }
}

// ---------------------------------------------------------------------------
// projection and stage combination
// ---------------------------------------------------------------------------
__device__ __forceinline__ void project_vjp(const double (&b)[12], const double (&yb)[12], double (&bb)[12]) {
    project_point_vjp(b, yb, bb);
}

// Final combination a = v0 + (dt/6)(((k1 + 2 k2) + 2 k3) + k4), u' = P(a):
// from ubar' (in adj) writes abar to v0bar and to abar; the stage RHS
// adjoints are (dt/6){1,2,2,1} abar plus the stage terms, formed later.
__global__ void __launch_bounds__(kThreads)
k_adj_final(const double* __restrict__ v0, const double* __restrict__ k1, const double* __restrict__ k2,
            const double* __restrict__ k3, const double* __restrict__ k4, const double* __restrict__ adj,
            double* __restrict__ v0bar, double* __restrict__ abar, Geo G, Box B) {
    Pt c;
    if (!owned_point(G, B, c)) return;
    const long long cs = G.cs, p = c.p;
    const double h6 = G.dt / 6.0;
    double b[12], yb[12], bb[12];
#pragma unroll
    for (int s = 0; s < 12; ++s) {
        const int f = s < 6 ? GXX + s : AXX + (s - 6);
        const long long q = f * cs + p;
        b[s] = v0[q] + h6 * (((k1[q] + 2.0 * k2[q]) + 2.0 * k3[q]) + k4[q]);
        yb[s] = adj[q];
    }
    project_vjp(b, yb, bb);
#pragma unroll
    for (int f = 0; f < NCOMP; ++f) {
        const long long q = f * cs + p;
        const int s = f < 6 ? f : ((f >= AXX && f <= AZZ) ? 6 + (f - AXX) : -1);
        const double a = s >= 0 ? bb[s] : adj[q];
        v0bar[q] = a;
        abar[q] = a;
    }
}

// Stage v = P(v0 + h k): from vbar adds bbar to v0bar and writes the
// adjoint of k, weight abar + h bbar (weight: k's factor in the final
// combination).
__global__ void __launch_bounds__(kThreads)
k_adj_stage(const double* __restrict__ v0, const double* __restrict__ k, double h, const double* __restrict__ vbar,
            double* __restrict__ v0bar, const double* __restrict__ abar, double weight, double* __restrict__ kbar,
            Geo G, Box B) {
    Pt c;
    if (!owned_point(G, B, c)) return;
    const long long cs = G.cs, p = c.p;
    double b[12], yb[12], bb[12];
#pragma unroll
    for (int s = 0; s < 12; ++s) {
        const int f = s < 6 ? GXX + s : AXX + (s - 6);
        const long long q = f * cs + p;
        b[s] = v0[q] + h * k[q];
        yb[s] = vbar[q];
    }
    project_vjp(b, yb, bb);
#pragma unroll
    for (int f = 0; f < NCOMP; ++f) {
        const long long q = f * cs + p;
        const int s = f < 6 ? f : ((f >= AXX && f <= AZZ) ? 6 + (f - AXX) : -1);
        const double a = s >= 0 ? bb[s] : vbar[q];
        v0bar[q] += a;
        kbar[q] = fma(h, a, weight * abar[q]);
    }
}

// Initial projection v0 = P(u): ubar = P^T v0bar (in place on the adjoint).
__global__ void __launch_bounds__(kThreads)
k_adj_initial(const double* __restrict__ u, const double* __restrict__ v0bar, double* __restrict__ adj, Geo G,
              Box B) {
    Pt c;
    if (!owned_point(G, B, c)) return;
    const long long cs = G.cs, p = c.p;
    double b[12], yb[12], bb[12];
#pragma unroll
    for (int s = 0; s < 12; ++s) {
        const int f = s < 6 ? GXX + s : AXX + (s - 6);
        b[s] = u[f * cs + p];
        yb[s] = v0bar[f * cs + p];
    }
    project_vjp(b, yb, bb);
#pragma unroll
    for (int f = 0; f < NCOMP; ++f) {
        const int s = f < 6 ? f : ((f >= AXX && f <= AZZ) ? 6 + (f - AXX) : -1);
        adj[f * cs + p] = s >= 0 ? bb[s] : v0bar[f * cs + p];
    }
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
struct Plan {
    Geo G;
    Box B;
    long long cs;        // component stride of a batch state
    size_t state;        // doubles per batch state (21 * cs)
    int steps, segment, nseg, store;
    // Segment j holds len(j) steps, in order: the first takes the remainder,
    // so the last -- recorded by the forward pass when stages are stored --
    // is a full one.
    int len(int j) const { return j == 0 ? steps - (nseg - 1) * segment : segment; }
};

int validate(const BssnParams* p, const char* where) {
    int st = validate_params(p);
    if (st) return st;
    for (int d = 0; d < 3; ++d)
        if (p->bc[2 * d] != p->bc[2 * d + 1])
            return fail(BSSN_ERR_INVALID,
                        std::string(where) + ": the adjoint needs both faces of an axis periodic or both Sommerfeld");
    if (p->kappa != 0.0) return fail(BSSN_ERR_INVALID, std::string(where) + ": the adjoint needs kappa = 0");
    if (p->precision != BSSN_PRECISION_F64)
        return fail(BSSN_ERR_INVALID, std::string(where) + ": the adjoint runs in FP64 arithmetic");
    return BSSN_OK;
}

int make_plan(const BssnPatch* patch, int32_t ninst, const BssnParams* params, int32_t steps, int32_t segment,
              int32_t store, const char* where, Plan& P) {
    int st = validate(params, where);
    if (st) return st;
    if (!patch || patch->ghost < 4) return fail(BSSN_ERR_INVALID, std::string(where) + ": patch ghost must be >= 4");
    if (ninst < 1) return fail(BSSN_ERR_INVALID, std::string(where) + ": instance count must be positive");
    if (steps < 0) return fail(BSSN_ERR_INVALID, std::string(where) + ": steps must be non-negative");
    int S[3], org[3], Pd[3];
    for (int d = 0; d < 3; ++d) {
        if (patch->n[d] < 8) return fail(BSSN_ERR_INVALID, std::string(where) + ": the adjoint needs 8+ samples per axis");
        S[d] = patch->n[d];
        org[d] = patch->ghost;
        Pd[d] = patch->n[d] + 2 * patch->ghost;
    }
    BssnParams q = *params;
    q.guard_cells = 0;
    for (int d = 0; d < 3; ++d) { q.owned_shape[d] = -1; q.reduced_axes[d] = 0; }
    for (int f = 0; f < 6; ++f) q.owned_faces[f] = 1;
    if ((st = make_geo(&q, S, org, Pd, P.G))) return st;
    P.G.ninst = ninst;
    P.G.istride = P.G.cs;
    P.G.cs *= ninst;
    P.cs = P.G.cs;
    P.state = (size_t)NCOMP * (size_t)P.cs;
    P.B = box_of(P.G);
    P.steps = steps;
    P.segment = segment > 0 ? segment : (steps > 0 ? (int)std::ceil(std::sqrt((double)steps)) : 1);
    if (P.segment > (steps > 0 ? steps : 1)) P.segment = steps > 0 ? steps : 1;
    P.nseg = steps > 0 ? (steps + P.segment - 1) / P.segment : 0;
    P.store = store < 0 ? 0 : (store > 2 ? 2 : store);
    return BSSN_OK;
}

// Work buffers of one RHS VJP (in units of cs): coefficients and the
// inner-derivative / folded-coefficient blocks.
constexpr size_t kVjpBlocks = NCOEF + 3 * NMIX;

struct Layout {
    double* ckpt;      // nseg states
    double* seg;       // segment states (step starts)
    double* segk;      // store >= 1: segment x 4 stage RHS states
    double* segv;      // store == 2: segment x 4 stage states (ghost-filled)
    double* V[4];      // stage states (ghost-filled)
    double* K[4];      // stage RHS values (recompute mode)
    double* KB[4];     // stage RHS adjoints
    double* v0bar;
    double* vb;
    double* acc;
    double* coef;      // NCOEF blocks
    double* d1;        // 3 NMIX blocks: inner derivatives, then the folded coefficients
    size_t doubles;
};

Layout layout_of(const Plan& P, double* base) {
    Layout L;
    double* q = base;
    auto take = [&](size_t n) { double* r = q; q += n; return r; };
    L.ckpt = take(P.nseg * P.state);
    L.seg = take((size_t)P.segment * P.state);
    L.segk = take(P.store ? (size_t)P.segment * 4 * P.state : 0);
    L.segv = take(P.store == 2 ? (size_t)P.segment * 4 * P.state : 0);
    for (int i = 0; i < 4; ++i) L.V[i] = take(P.state);
    for (int i = 0; i < 4; ++i) L.K[i] = P.store ? nullptr : take(P.state);
    for (int i = 0; i < 4; ++i) L.KB[i] = take(P.state);
    L.v0bar = take(P.state);
    L.vb = take(P.state);
    L.acc = take(P.state);
    L.coef = take((size_t)NCOEF * P.cs);
    L.d1 = take((size_t)3 * NMIX * P.cs);
    L.doubles = (size_t)(q - base);
    return L;
}

cudaError_t fill(double* a, int ncomp, const Geo& G, cudaStream_t s) { return launch_fill_periodic(a, ncomp, G, s); }

// Stage RHS values and stage states of segment step n (the working buffers
// when the mode does not keep them).
void step_buffers(const Layout& L, const Plan& P, int n, double* K[4], double* V[4]) {
    for (int i = 0; i < 4; ++i) {
        K[i] = P.store ? L.segk + ((size_t)n * 4 + i) * P.state : L.K[i];
        V[i] = P.store == 2 ? L.segv + ((size_t)n * 4 + i) * P.state : L.V[i];
    }
}

// RHS VJP: ubar (= or +=) (dRHS/du)^T kbar at state u; u and kbar ghost-filled.
template <bool Closed>
cudaError_t rhs_vjp_form(const double* u, const double* kbar, double kscale, double* ubar, int accumulate,
                         double* coef, double* d1, const Geo& G, const Box& B, cudaStream_t s) {
    cudaError_t e = launch_inner_derivs(u, d1, G, B, s);
    if (e != cudaSuccess) return e;
    const unsigned nb = blocks_of(box_threads(G, B));
    BSSN_LAUNCH(KC_ADJ_POINT, k_adj_point<Closed>, nb, kThreads, s, u, d1, kbar, kscale, ubar, coef, G, B,
                point_params(G), accumulate);
    // Stencils read the neighbours of the first-derivative coefficients of K
    // and Gt (blocks 24..26 and 36..44) and of every second-derivative
    // coefficient (45..110); the NMIX fields' first-derivative coefficients
    // are read at their own point only.
    if ((e = fill(coef + (long long)(I_DK - 21) * G.cs, 3, G, s)) != cudaSuccess) return e;
    if ((e = fill(coef + (long long)(I_DGT - 21) * G.cs, NCOEF - (I_DGT - 21), G, s)) != cudaSuccess) return e;
    BSSN_LAUNCH(KC_ADJ_STENCIL, k_adj_mixed<Closed>, nb, kThreads, s, coef, d1, G, B);
    if constexpr (Closed) BSSN_LAUNCH(KC_ADJ_STENCIL, k_adj_band_mixed, nb, kThreads, s, coef, d1, G, B);
    if ((e = fill(d1, 3 * NMIX, G, s)) != cudaSuccess) return e;
    BSSN_LAUNCH(KC_ADJ_STENCIL, k_adj_field<Closed>, nb, kThreads, s, u, kbar, kscale, coef, d1, ubar, G, B);
    if constexpr (Closed) {
        BSSN_LAUNCH(KC_ADJ_STENCIL, k_adj_band_field, nb, kThreads, s, u, kbar, kscale, coef, d1, ubar, G, B);
        BSSN_LAUNCH(KC_ADJ_STENCIL, k_adj_sommerfeld, nb, kThreads, s, kbar, kscale, ubar, G, B);
    }
    return cudaGetLastError();
}
cudaError_t rhs_vjp(const double* u, const double* kbar, double kscale, double* ubar, int accumulate, double* coef,
                    double* d1, const Geo& G, const Box& B, cudaStream_t s) {
    return G.any_sommerfeld ? rhs_vjp_form<true>(u, kbar, kscale, ubar, accumulate, coef, d1, G, B, s)
                            : rhs_vjp_form<false>(u, kbar, kscale, ubar, accumulate, coef, d1, G, B, s);
}

// One forward RK4 step from u_n (owned values) recording the stage states V
// (ghost-filled) and the stage RHS values K; the new state goes to next.
// The kernels and their order are the production step's, so the recorded
// values are the forward's own.
cudaError_t record_step(const double* un, double* const V[4], double* const K[4], double* acc, double* next,
                        double* d1, const Plan& P, cudaStream_t s) {
    const Geo& G = P.G;
    const Box& B = P.B;
    RhsWork w;
    w.d1 = d1;
    cudaError_t e = cudaMemcpyAsync(V[0], un, P.state * sizeof(double), cudaMemcpyDeviceToDevice, s);
    if (e == cudaSuccess) e = launch_project(V[0], G, B, s);
    for (int i = 0; i < 4 && e == cudaSuccess; ++i) {
        if ((e = fill(V[i], NCOMP, G, s)) != cudaSuccess) break;
        if ((e = launch_rhs(V[i], K[i], w, G, B, s)) != cudaSuccess) break;
        double* out = i < 3 ? V[i + 1] : next;
        e = launch_rk4_stage(V[0], K[i], acc, out, G, B, i + 1, G.dt, 0, 1, s);
    }
    return e;
}

// The stage states of a recorded step from u_n and its stage RHS values.
cudaError_t replay_stages(const double* un, double* const K[4], double* const V[4], double* acc, const Plan& P,
                          cudaStream_t s) {
    const Geo& G = P.G;
    const Box& B = P.B;
    cudaError_t e = cudaMemcpyAsync(V[0], un, P.state * sizeof(double), cudaMemcpyDeviceToDevice, s);
    if (e == cudaSuccess) e = launch_project(V[0], G, B, s);
    if (e == cudaSuccess) e = fill(V[0], NCOMP, G, s);
    for (int i = 1; i < 4 && e == cudaSuccess; ++i) {
        e = launch_rk4_stage(V[0], K[i - 1], acc, V[i], G, B, i, G.dt, 0, 1, s);
        if (e == cudaSuccess) e = fill(V[i], NCOMP, G, s);
    }
    return e;
}

// Reverse of one RK4 step: adj holds ubar_{n+1} on entry and ubar_n on exit.
cudaError_t backward_step(const double* un, double* const V[4], double* const K[4], double* adj, const Layout& L,
                          const Plan& P, cudaStream_t s) {
    const Geo& G = P.G;
    const Box& B = P.B;
    const unsigned nb = blocks_of(box_threads(G, B));
    // abar lives in KB[3]; the adjoints of k1..k3 go to KB[0..2]
    double* abar = L.KB[3];
    BSSN_LAUNCH(KC_ADJ_STAGE, k_adj_final, nb, kThreads, s, V[0], K[0], K[1], K[2], K[3], adj, L.v0bar, abar, G, B);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = fill(abar, NCOMP, G, s);
    // k4's adjoint is (dt/6) abar: the VJP scales abar as it reads it
    const double h[3] = {0.5 * G.dt, 0.5 * G.dt, G.dt};
    const double weight[3] = {G.dt / 6.0, G.dt / 3.0, G.dt / 3.0};   // of k1, k2, k3 in the final combination
    for (int i = 3; i >= 1 && e == cudaSuccess; --i) {
        // V[i] = P(V[0] + h[i-1] K[i-1]); its RHS is K[i]
        const double* kin = i == 3 ? abar : L.KB[i];
        const double scale = i == 3 ? G.dt / 6.0 : 1.0;
        if ((e = rhs_vjp(V[i], kin, scale, L.vb, 0, L.coef, L.d1, G, B, s)) != cudaSuccess) break;
        BSSN_LAUNCH(KC_ADJ_STAGE, k_adj_stage, nb, kThreads, s, V[0], K[i - 1], h[i - 1], L.vb, L.v0bar, abar,
                    weight[i - 1], L.KB[i - 1], G, B);
        e = cudaGetLastError();
        if (e == cudaSuccess) e = fill(L.KB[i - 1], NCOMP, G, s);
    }
    if (e == cudaSuccess) e = rhs_vjp(V[0], L.KB[0], 1.0, L.v0bar, 1, L.coef, L.d1, G, B, s);
    if (e == cudaSuccess) {
        BSSN_LAUNCH(KC_ADJ_STAGE, k_adj_initial, nb, kThreads, s, un, L.v0bar, adj, G, B);
        e = cudaGetLastError();
    }
    return e;
}

}  // namespace
}  // namespace adjoint
}  // namespace bssn

using namespace bssn;
using namespace bssn::adjoint;

extern "C" {

size_t bssn_rhs_vjp_workspace_bytes(const BssnPatch* patch, int32_t ninst) {
    if (!patch || ninst < 1) return 0;
    size_t block = 1;
    for (int d = 0; d < 3; ++d) block *= (size_t)(patch->n[d] + 2 * patch->ghost);
    return kVjpBlocks * (size_t)ninst * block * sizeof(double);
}

int bssn_rhs_vjp(double* states, double* rhs_adjoint, double* state_adjoint, const BssnPatch* patch, int32_t ninst,
                 const BssnParams* params, void* workspace, size_t workspace_bytes, void* stream) {
    if (!states || !rhs_adjoint || !state_adjoint) return fail(BSSN_ERR_INVALID, "bssn_rhs_vjp: null pointer");
    Plan P;
    int st = make_plan(patch, ninst, params, 0, 1, 0, "bssn_rhs_vjp", P);
    if (st) return st;
    if (!workspace || workspace_bytes < bssn_rhs_vjp_workspace_bytes(patch, ninst))
        return fail(BSSN_ERR_WORKSPACE, "bssn_rhs_vjp: workspace missing or smaller than bssn_rhs_vjp_workspace_bytes");
    cudaStream_t s = (cudaStream_t)stream;
    double* coef = (double*)workspace;
    double* d1 = coef + (size_t)NCOEF * P.cs;
    cudaError_t e = fill(states, NCOMP, P.G, s);
    if (e == cudaSuccess) e = fill(rhs_adjoint, NCOMP, P.G, s);
    if (e == cudaSuccess) e = rhs_vjp(states, rhs_adjoint, 1.0, state_adjoint, 0, coef, d1, P.G, P.B, s);
    return cuda_status(e, "bssn_rhs_vjp");
}

size_t bssn_adjoint_workspace_bytes(const BssnPatch* patch, int32_t ninst, const BssnParams* params, int32_t steps,
                                    int32_t segment, int32_t store_stages) {
    Plan P;
    if (make_plan(patch, ninst, params, steps, segment, store_stages, "bssn_adjoint_workspace_bytes", P)) return 0;
    return layout_of(P, nullptr).doubles * sizeof(double);
}

int bssn_adjoint_forward(double* states, const BssnPatch* patch, int32_t ninst, const BssnParams* params,
                         int32_t steps, int32_t segment, int32_t store_stages, void* workspace, size_t workspace_bytes,
                         void* stream) {
    if (!states) return fail(BSSN_ERR_INVALID, "bssn_adjoint_forward: null pointer");
    Plan P;
    int st = make_plan(patch, ninst, params, steps, segment, store_stages, "bssn_adjoint_forward", P);
    if (st) return st;
    const Layout L = layout_of(P, (double*)workspace);
    if (!workspace || workspace_bytes < L.doubles * sizeof(double))
        return fail(BSSN_ERR_WORKSPACE, "bssn_adjoint_forward: workspace smaller than bssn_adjoint_workspace_bytes");
    cudaStream_t s = (cudaStream_t)stream;
    RhsWork w;
    w.d1 = L.d1;
    cudaError_t e = cudaSuccess;
    for (int j = 0; j < P.nseg && e == cudaSuccess; ++j) {
        e = cudaMemcpyAsync(L.ckpt + (size_t)j * P.state, states, P.state * sizeof(double), cudaMemcpyDeviceToDevice, s);
        const int len = P.len(j);
        if (P.store && j == P.nseg - 1) {
            // the last segment is recorded now (step starts and stage RHS
            // values), so the backward pass starts without re-running it
            for (int n = 0; n < len && e == cudaSuccess; ++n) {
                double* un = L.seg + (size_t)n * P.state;
                e = cudaMemcpyAsync(un, states, P.state * sizeof(double), cudaMemcpyDeviceToDevice, s);
                double *K[4], *V[4];
                step_buffers(L, P, n, K, V);
                if (e == cudaSuccess) e = record_step(un, V, K, L.acc, states, L.d1, P, s);
            }
            break;
        }
        for (int n = 0; n < len && e == cudaSuccess; ++n) {
            e = launch_project(states, P.G, P.B, s);
            if (e == cudaSuccess) e = rk4_step_patch(states, L.V[0], L.V[1], L.acc, w, P.G, P.B, true, 0, s);
        }
    }
    return cuda_status(e, "bssn_adjoint_forward");
}

int bssn_adjoint_backward(double* adjoint, const BssnPatch* patch, int32_t ninst, const BssnParams* params,
                          int32_t steps, int32_t segment, int32_t store_stages, void* workspace, size_t workspace_bytes,
                          void* stream) {
    if (!adjoint) return fail(BSSN_ERR_INVALID, "bssn_adjoint_backward: null pointer");
    Plan P;
    int st = make_plan(patch, ninst, params, steps, segment, store_stages, "bssn_adjoint_backward", P);
    if (st) return st;
    const Layout L = layout_of(P, (double*)workspace);
    if (!workspace || workspace_bytes < L.doubles * sizeof(double))
        return fail(BSSN_ERR_WORKSPACE, "bssn_adjoint_backward: workspace smaller than bssn_adjoint_workspace_bytes");
    cudaStream_t s = (cudaStream_t)stream;
    RhsWork w;
    w.d1 = L.d1;
    cudaError_t e = cudaSuccess;
    for (int j = P.nseg - 1; j >= 0 && e == cudaSuccess; --j) {
        const int len = P.len(j);
        // re-run the segment from its checkpoint, keeping step starts (and
        // stages); with stored stages the forward pass recorded the last one
        const bool recorded = P.store && j == P.nseg - 1;
        if (!recorded)
            e = cudaMemcpyAsync(L.seg, L.ckpt + (size_t)j * P.state, P.state * sizeof(double), cudaMemcpyDeviceToDevice,
                                s);
        for (int n = 0; !recorded && n + 1 < len + (P.store ? 1 : 0) && e == cudaSuccess; ++n) {
            double* un = L.seg + (size_t)n * P.state;
            if (P.store) {
                double *K[4], *V[4];
                step_buffers(L, P, n, K, V);
                double* next = n + 1 < len ? L.seg + (size_t)(n + 1) * P.state : L.vb;
                e = record_step(un, V, K, L.acc, next, L.d1, P, s);
            } else {
                double* next = L.seg + (size_t)(n + 1) * P.state;
                e = cudaMemcpyAsync(next, un, P.state * sizeof(double), cudaMemcpyDeviceToDevice, s);
                if (e == cudaSuccess) e = launch_project(next, P.G, P.B, s);
                if (e == cudaSuccess) e = rk4_step_patch(next, L.V[0], L.V[1], L.acc, w, P.G, P.B, true, 0, s);
            }
        }
        for (int n = len - 1; n >= 0 && e == cudaSuccess; --n) {
            double* un = L.seg + (size_t)n * P.state;
            double *K[4], *V[4];
            step_buffers(L, P, n, K, V);
            if (P.store == 1) e = replay_stages(un, K, V, L.acc, P, s);
            else if (P.store == 0) e = record_step(un, V, K, L.acc, L.vb, L.d1, P, s);
            if (e == cudaSuccess) e = backward_step(un, V, K, adjoint, L, P, s);
        }
    }
    return cuda_status(e, "bssn_adjoint_backward");
}

}  // extern "C"
