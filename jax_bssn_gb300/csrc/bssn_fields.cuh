// Component numbering, point addressing and pointwise tensor algebra.
//
// Pointwise algebra follows JAX_BSSN/bssn/tensor_algebra.py: the inverse
// conformal metric (:20-71), the closed-form 3x3 determinant (:74-96),
// Christoffel symbols (:148-193) and the trace-free part (:359-381).  The
// reference inverts by an explicit Cholesky factor; the RHS kernels invert by
// cofactors and one reciprocal of the determinant, which agrees to rounding
// (gt^ij only ever multiplies perturbation-sized derivatives there) and costs
// one FP64 reciprocal instead of three square roots and three reciprocals.  The algebraic projection (JAX_BSSN/evolution/time_evolve.py:94-141)
// is written with round-to-nearest intrinsics in the reference's operation
// order and a correctly rounded det^(-1/3), so a projected conformal metric is
// bit-identical to the float64 reference: that matters because its second
// derivatives enter the Ricci tensor with a 1/dx^2 gain on any last-bit
// difference.
#pragma once

#include "bssn_stencil.cuh"

namespace bssn {

enum Comp {
    GXX = 0, GXY, GXZ, GYY, GYZ, GZZ, CW,
    AXX, AXY, AXZ, AYY, AYZ, AZZ, CK,
    GTX, GTY, GTZ, CALPHA, BX, BY, BZ, NCOMP
};

__host__ __device__ constexpr int sym(int i, int j) {
    return (i == j) ? (i == 0 ? 0 : (i == 1 ? 3 : 5))
                    : ((i + j == 1) ? 1 : ((i + j == 2) ? 2 : 4));
}

// Fields whose first derivatives are stored for composed mixed second
// derivatives: gt (6), W, alpha, beta (3).
constexpr int NMIX = 11;
constexpr int MIX_G = 0, MIX_W = 6, MIX_ALPHA = 7, MIX_B = 8;
__host__ __device__ constexpr int mix_source(int f) {
    return f < 6 ? GXX + f : (f == 6 ? CW : (f == 7 ? CALPHA : BX + (f - 8)));
}

// Fields whose first derivatives are stored when kappa != 0 for the
// momentum-constraint derivative: At (6), K, B_i^j (9) -- the latter from the
// derived-field buffer.  Indexed after the NMIX base set.
constexpr int NMIX_MOM = 16;

// Compute box: linear thread index -> padded (x, y, z).  `fast` names the
// fastest-varying axis: z (2, the default and the memory order), y (1, then z,
// then x) or x (0, then z, then y).  Shell slabs thin in z or y run with
// another fast axis so that the samples of a warp share their closure rows.
struct Box {
    int lo[3];
    int n[3];
    long long count;
    int fast = 2;
    // z fastest (interior boxes always are)
    __device__ __forceinline__ void coords_z(long long t, int (&ix)[3]) const {
        const long long yz = (long long)n[1] * n[2];
        const int x = (int)(t / yz);
        const long long r = t - (long long)x * yz;
        const int y = (int)(r / n[2]);
        ix[0] = lo[0] + x;
        ix[1] = lo[1] + y;
        ix[2] = lo[2] + (int)(r - (long long)y * n[2]);
    }
    __device__ __forceinline__ void coords(long long t, int (&ix)[3]) const {
        if (fast == 2) {
            coords_z(t, ix);
            return;
        }
        // fast = 1: order (x, z, y); fast = 0: order (y, z, x) -- z is the middle axis
        const int nc = n[fast];
        const long long bc = (long long)n[2] * nc;
        const int ia = (int)(t / bc);
        const long long r = t - (long long)ia * bc;
        const int ib = (int)(r / nc);
        const int ic = (int)(r - (long long)ib * nc);
        ix[2] = lo[2] + ib;
        if (fast == 1) { ix[0] = lo[0] + ia; ix[1] = lo[1] + ic; }
        else { ix[1] = lo[1] + ia; ix[0] = lo[0] + ic; }
    }
};

__device__ __forceinline__ long long lin(const Geo& G, const int (&ix)[3]) {
    return (long long)ix[0] * G.st[0] + (long long)ix[1] * G.st[1] + ix[2];
}

// Threads of a launch over box B: count per instance times the instances.
__host__ __device__ __forceinline__ long long box_threads(const Geo& G, const Box& B) {
    return B.count * G.ninst;
}

// Split a launch's linear thread index into the index within one instance's
// box (t, updated) and that instance's sample offset (returned).
__device__ __forceinline__ long long instance_offset(const Geo& G, const Box& B, long long& t) {
    if (G.ninst == 1) return 0;
    const long long i = t / B.count;
    t -= i * B.count;
    return i * G.istride;
}

// ---------------------------------------------------------------------------
// inverse metric by cofactors over the determinant, FMA allowed; a template on
// the arithmetic type (the reciprocal in that type)
// ---------------------------------------------------------------------------
template <typename R>
__device__ __forceinline__ void inverse_metric(const R (&g)[6], R (&gi)[6]) {
    const R c00 = g[3] * g[5] - g[4] * g[4];
    const R c01 = g[2] * g[4] - g[1] * g[5];
    const R c02 = g[1] * g[4] - g[2] * g[3];
    const R r = R(1) / (g[0] * c00 + g[1] * c01 + g[2] * c02);
    gi[0] = c00 * r;
    gi[1] = c01 * r;
    gi[2] = c02 * r;
    gi[3] = (g[0] * g[5] - g[2] * g[2]) * r;
    gi[4] = (g[1] * g[2] - g[0] * g[4]) * r;
    gi[5] = (g[0] * g[3] - g[1] * g[1]) * r;
}

// Correctly rounded a/6, the final RK4 division of the reference
// (time_evolve.py:144-217), in three FP64 operations by Markstein's theorem
// (P. Markstein, IBM J. Res. Dev. 34(1), 1990, 111-119): y = RN(1/6) is within
// half an ulp of 1/6 and q = RN(a*y) within one ulp of a/6, so the remainder
// r = a - 6q is exact under an FMA and RN(q + r*y) = RN(a/6).  The theorem
// assumes no underflow or overflow; outside that range, and for zeros, infinities
// and NaN, the hardware division is used.
__device__ __forceinline__ double div6_rn(double a) {
    const double m = fabs(a);
    if (!(m >= 0x1p-960 && m <= 0x1p1020)) return __ddiv_rn(a, 6.0);
    constexpr double y = 1.0 / 6.0;
    const double q = __dmul_rn(a, y);
    const double r = __fma_rn(-6.0, q, a);
    return __fma_rn(r, y, q);
}

// The reference's Cholesky factorisation (tensor_algebra.py:20-71) with every
// operation rounded in its order (used by the projection, whose output is part
// of the state).
__device__ __forceinline__ void inverse_metric_rn(const double (&g)[6], double (&gi)[6]) {
    const double l00 = __dsqrt_rn(g[0]);
    const double l10 = __ddiv_rn(g[1], l00);
    const double l20 = __ddiv_rn(g[2], l00);
    const double l11 = __dsqrt_rn(__dadd_rn(g[3], -__dmul_rn(l10, l10)));
    const double l21 = __ddiv_rn(__dadd_rn(g[4], -__dmul_rn(l20, l10)), l11);
    const double l22 = __dsqrt_rn(__dadd_rn(__dadd_rn(g[5], -__dmul_rn(l20, l20)), -__dmul_rn(l21, l21)));
    const double m00 = __ddiv_rn(1.0, l00);
    const double m10 = __ddiv_rn(-l10, __dmul_rn(l00, l11));
    const double m11 = __ddiv_rn(1.0, l11);
    const double m20 = __ddiv_rn(__dadd_rn(__dmul_rn(l10, l21), -__dmul_rn(l20, l11)),
                                 __dmul_rn(__dmul_rn(l00, l11), l22));
    const double m21 = __ddiv_rn(-l21, __dmul_rn(l11, l22));
    const double m22 = __ddiv_rn(1.0, l22);
    gi[0] = __dadd_rn(__dadd_rn(__dmul_rn(m00, m00), __dmul_rn(m10, m10)), __dmul_rn(m20, m20));
    gi[1] = __dadd_rn(__dmul_rn(m10, m11), __dmul_rn(m20, m21));
    gi[2] = __dmul_rn(m20, m22);
    gi[3] = __dadd_rn(__dmul_rn(m11, m11), __dmul_rn(m21, m21));
    gi[4] = __dmul_rn(m21, m22);
    gi[5] = __dmul_rn(m22, m22);
}

// Closed-form determinant of a symmetric 3x3 (six Sarrus products, fixed order).
__device__ __forceinline__ double det_sym_rn(const double (&g)[6]) {
    // g00 g11 g22 + g01 g12 g20 + g02 g10 g21 - g02 g11 g20 - g00 g12 g21 - g01 g10 g22
    double acc = __dmul_rn(__dmul_rn(g[0], g[3]), g[5]);
    acc = __dadd_rn(acc, __dmul_rn(__dmul_rn(g[1], g[4]), g[2]));
    acc = __dadd_rn(acc, __dmul_rn(__dmul_rn(g[2], g[1]), g[4]));
    acc = __dadd_rn(acc, -__dmul_rn(__dmul_rn(g[2], g[3]), g[2]));
    acc = __dadd_rn(acc, -__dmul_rn(__dmul_rn(g[0], g[4]), g[4]));
    acc = __dadd_rn(acc, -__dmul_rn(__dmul_rn(g[1], g[1]), g[5]));
    return acc;
}

// ---------------------------------------------------------------------------
// Correctly rounded x^(-1/3) for x > 0 (the projection's det^(-1/3)).
//
// Near x = 1 -- where every projected metric's determinant sits, often on
// values like 1 - 3*2^-53 whose cube root lies within 2^-106 of a rounding
// midpoint -- the result is decided by exact midpoint tests.  Elsewhere
// rcbrt() gives y within a couple of ulp; one Newton step for y^-3 = x carried
// in double-double (Dekker/Knuth error-free transformations) gives ~100 bits,
// and the final rounding of the double-double sum yields the correctly
// rounded result except within ~2^-100 of a rounding midpoint.  The float64
// reference evaluates pow(det, -1.0/3.0); the double exponent exceeds -1/3 by
// kPowThirdOffset, so the result is x^(-1/3) * (1 + kPowThirdOffset*ln x),
// folded into the same correction before the single final rounding.
// ---------------------------------------------------------------------------
constexpr double kPowThirdOffset = 1.850371707708594e-17;

__device__ __forceinline__ void two_prod(double a, double b, double& p, double& e) {
    p = a * b;
    e = fma(a, b, -p);
}
__device__ __forceinline__ void two_sum(double a, double b, double& s, double& e) {
    s = a + b;
    const double bb = s - a;
    e = (a - (s - bb)) + (b - bb);
}

// Is y* = pow(x, -1/3 + kPowThirdOffset) above the midpoint m = 1 + mu, for
// x = 1 + xi with |xi| < 2^-28?  y* > m  <=>  x m^3 - 1 < 3*offset*ln x.  xi and
// mu are exact multiples of 2^-54, and x m^3 - 1 = (xi + 3 mu) + 3 mu (mu + xi)
// + mu^2 (mu + 3 xi) + xi mu^3, whose first term is either exactly zero or at
// least 2^-54 while the rest stay below 2^-55: the comparison is exact.
__device__ __forceinline__ bool cbrt_above_midpoint(double xi, double mu) {
    const double a1 = xi + 3.0 * mu;  // exact: both multiples of 2^-54 with few bits
    if (a1 != 0.0) return a1 < 0.0;
    double ph, pl;
    two_prod(3.0 * mu, mu + xi, ph, pl);  // mu + xi and 3 mu are exact
    const double a3 = mu * mu * (mu + 3.0 * xi);
    const double f = 3.0 * kPowThirdOffset * (xi - 0.5 * xi * xi);
    return ((ph - f) + (pl + a3)) < 0.0;
}

__device__ __forceinline__ double inv_cbrt_cr(double x) {
    if (!(x > 0.0) || isinf(x)) return pow(x, -1.0 / 3.0);
    const double xi = x - 1.0;
    if (fabs(xi) < 0x1p-28) {
        // Near one (every projected metric): pick the correctly rounded double
        // by exact midpoint tests around a first-order candidate.  Below
        // 2^-28 the candidate is within two ulp and the first-order term of
        // the midpoint test is either zero or larger than all the others.
        double y = 1.0 - xi * (1.0 / 3.0);
#pragma unroll 1
        for (int it = 0; it < 4; ++it) {
            const double up = nextafter(y, 2.0);
            if (cbrt_above_midpoint(xi, (y - 1.0) + 0.5 * (up - y))) { y = up; continue; }
            const double dn = nextafter(y, 0.0);
            if (!cbrt_above_midpoint(xi, (y - 1.0) - 0.5 * (y - dn))) { y = dn; continue; }
            break;
        }
        return y;
    }
    double y = rcbrt(x);
    // r = 1 - x*y^3 in double-double, then y' = y + y*r/3.
    double y2h, y2l;
    two_prod(y, y, y2h, y2l);
    double y3h, y3l;
    two_prod(y2h, y, y3h, y3l);
    y3l = fma(y2l, y, y3l);
    double xyh, xyl;
    two_prod(x, y3h, xyh, xyl);
    xyl = fma(x, y3l, xyl);
    double rh, rl;
    two_sum(1.0, -xyh, rh, rl);
    rl -= xyl;
    const double r = rh + rl;
    // correction c = y * (r/3 + offset*ln x), added to y then rounded once
    const double c = y * (r * (1.0 / 3.0) + kPowThirdOffset * log(x));
    double sh, sl;
    two_sum(y, c, sh, sl);
    return sh + sl;
}

// ---------------------------------------------------------------------------
// Christoffel symbols from dg[k][sym(i,j)] = d_k g_ij
//   c1[i][sym(j,k)] = Gamma_ijk = (d_k g_ij + d_j g_ik - d_i g_jk)/2
//   c2[i][sym(j,k)] = Gamma^i_jk = g^im Gamma_mjk
// ---------------------------------------------------------------------------
template <typename R>
__device__ __forceinline__ void christoffel_first(const R (&dg)[3][6], R (&c1)[3][6]) {
    // Index patterns whose terms cancel are written out: Gamma_iii = d_i g_ii / 2,
    // Gamma_ijj = d_j g_ij - d_i g_jj / 2, Gamma_iik = Gamma_iki = d_k g_ii / 2.
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j)
#pragma unroll
            for (int k = j; k < 3; ++k) {
                R v;
                if (j == k && i == j) v = R(0.5) * dg[i][sym(i, i)];
                else if (j == k) v = dg[j][sym(i, j)] + R(-0.5) * dg[i][sym(j, j)];
                else if (i == j) v = R(0.5) * dg[k][sym(i, i)];
                else if (i == k) v = R(0.5) * dg[j][sym(i, i)];
                else v = R(0.5) * (dg[k][sym(i, j)] + dg[j][sym(i, k)] - dg[i][sym(j, k)]);
                c1[i][sym(j, k)] = v;
            }
}
template <typename R>
__device__ __forceinline__ void christoffel(const R (&dg)[3][6], const R (&gi)[6], R (&c1)[3][6], R (&c2)[3][6]) {
    christoffel_first(dg, c1);
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int s = 0; s < 6; ++s)
            c2[i][s] = gi[sym(i, 0)] * c1[0][s] + gi[sym(i, 1)] * c1[1][s] + gi[sym(i, 2)] * c1[2][s];
}

}  // namespace bssn
