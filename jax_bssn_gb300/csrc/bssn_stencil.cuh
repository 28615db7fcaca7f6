// Device-side finite-difference stencils of the BSSN hot path (sm_103a).
//
// Operators follow the reference's definitions (uwplasma/JAX_BSSN):
//   centred D1, MAD blend, closures    JAX_BSSN/evolution/derivatives.py:42-163
//   upwind D1 (D4/D6, MAD, faces)      JAX_BSSN/evolution/derivatives.py:166-338
//   pure D2, MAD blend, closures       JAX_BSSN/evolution/derivatives.py:341-461
//   sixth difference, closures         JAX_BSSN/evolution/derivatives.py:463-599
//   KO dissipation                     JAX_BSSN/evolution/spatial_derivatives.py:81-92
//
// Every stencil reads a field through a pointer to the sample at the point and
// the stride of the axis, so one code path serves x, y and z.
//
// The stencils are templates on the arithmetic type R.  R = double is the
// plain FP64 form: numerators whose terms cancel (D2, upwind, the sixth
// difference and all one-sided closures) are accumulated with explicit
// round-to-nearest intrinsics in the reference's term order, so the compiler
// cannot contract them into FMAs and their rounding matches the float64
// reference bit for bit (it is not amplified by the 1/dx^2 scaling).  A term
// whose coefficient is +-1 or an upward power of two is an exact product, so
// it is added by a plain add or a fused multiply-add with the same bits.
// Centred differences of neighbouring pairs carry no such amplification, and
// neither does anything after a numerator is formed (its scaling by 1/dx, the
// shift factor of the advection term, the KO factor and the sum over axes):
// those are left free for FMA contraction and regrouping.  R = float is the FP32-arithmetic form: the same
// operators on float samples (perturbations about a constant background),
// with every coefficient taken in float so no FP64 instruction is issued, and
// contraction allowed throughout.  Float numerators of operators whose
// coefficients sum to zero (D2, the sixth difference, every closure) are
// formed from differences to the centre sample, f(k) - f(0): a float sum of
// like samples rounds at eps*|f|, which the 1/dx^2 scaling would turn into
// noise far above the operator's value for a small, smooth perturbation,
// while the differences round at eps times themselves.
#pragma once

#include <cstdint>
#include <type_traits>

namespace bssn {

constexpr int kSommerfeld = 1;
constexpr int kPrecisionF64 = 0;   // plain FP64 arithmetic
constexpr int kPrecisionF32 = 1;   // FP32 RHS arithmetic, FP64 state and RK4
constexpr int kPrecisionF32Paired = 2;   // the same, second-derivative inputs as float pairs
// Every form but the plain FP64 one runs the float kernels.
__host__ __device__ constexpr bool float_form(int precision) { return precision != kPrecisionF64; }

// One axis of a padded patch: extent, compute range, closure range and the
// face/MAD policy for this array (JAX_BSSN/evolution/spatial_derivatives.py:18-41).
struct Axis {
    int P;            // padded extent
    int lo, hi;       // compute range [lo, hi) in padded indices
    int start, end;   // owned range [start, end) where face closures apply
    int lbc, rbc;     // 1: Sommerfeld closure at the lower/upper owned face
    int reduced;      // derivatives along this axis are identically zero
    int mad;          // 1: blend q*D4 + (1-q)*D6 (periodic axes with q != 1)
    int slo, shi;     // 1: Sommerfeld RHS replacement on the lower/upper owned face
    int org;          // padded index of array index 0 (coordinates and closures)
    double q, omq;    // q and 1 - q
    double xmin;      // coordinate of array index 0: x = xmin + dx * (i - org)
    float fq, fomq;   // q and 1 - q in float (FP32-arithmetic form)
};

// Float copies of the scalar coefficients (FP32-arithmetic form).
struct GeoF {
    float inv_dx, inv_12dx, inv_60dx, inv_12dx2, inv_dx2, inv_dx6h5, nu64, eta, kappa, g;
    float d1a, d1b, ko_scale;
};

// Per-launch geometry and scalar parameters (passed by value).
struct Geo {
    Axis ax[3];
    long long st[3];  // element strides of x, y, z
    long long cs;     // component stride (samples per padded block)
    double dx;
    double inv_dx;    // 1/dx
    double inv_12dx;  // 1/(12 dx)
    double inv_60dx;  // 1/(60 dx)
    double inv_12dx2; // 1/(12 dx^2)
    double inv_dx2;   // 1/dx^2
    double inv_dx6h5; // h^5 / dx^6 (KO factor on the undivided sixth difference)
    double nu64;      // nu / 64
    double d1a, d1b;  // 2/(3 dx) and -1/(12 dx): centred D4 weights of the pair differences
    double ko_scale;  // nu/64 * h^5/dx^6: KO factor on the summed sixth-difference numerators
    double eta, kappa, g, dt;
    int gauge, zero_shift;
    int any_sommerfeld;
    int precision;    // kPrecisionF64, kPrecisionF32 or kPrecisionF32Paired
    // Independent instances of the same patch in one launch: buffers are laid
    // out [component][instance][padded block], so cs = ninst * istride and an
    // instance starts istride samples after the previous one.
    int ninst;
    long long istride;
    GeoF gf;
};

// Pick the coefficient copy of the arithmetic type R.
template <typename R>
__host__ __device__ __forceinline__ R coef_pick(double d, float f) {
    if constexpr (std::is_same<R, float>::value) return f;
    else return d;
}
#define BSSN_CO(R, G, name) (::bssn::coef_pick<R>((G).name, (G).gf.name))
#define BSSN_AQ(R, a) (::bssn::coef_pick<R>((a).q, (a).fq))
#define BSSN_AOMQ(R, a) (::bssn::coef_pick<R>((a).omq, (a).fomq))

// Rounded sum and product of the arithmetic type: explicit round-to-nearest
// for double (no contraction), plain operators for float.
template <typename R> struct Num;
template <> struct Num<double> {
    static __device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }
    static __device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
};
template <> struct Num<float> {
    static __device__ __forceinline__ float add(float a, float b) { return a + b; }
    static __device__ __forceinline__ float mul(float a, float b) { return a * b; }
};

// |c| in {2, 4, ..., 64}: c*f is exact for every finite f that does not overflow.
__host__ __device__ constexpr bool upward_pow2(double c) {
    const double a = c < 0.0 ? -c : c;
    return a == 2.0 || a == 4.0 || a == 8.0 || a == 16.0 || a == 32.0 || a == 64.0;
}

// acc + c*f with the product and the sum each rounded (the reference's
// rounding).  c is a compile-time coefficient after inlining: +-1 needs no
// product, and an upward power of two makes the product exact, so one fused
// multiply-add returns the same bits as the rounded product and sum.
template <typename R>
__device__ __forceinline__ R mac(R acc, double c, R f) {
    if constexpr (std::is_same<R, double>::value) {
        if (c == 1.0) return __dadd_rn(acc, f);
        if (c == -1.0) return __dadd_rn(acc, -f);
        if (upward_pow2(c)) return __fma_rn(c, f, acc);
        return __dadd_rn(acc, __dmul_rn(c, f));
    } else {
        return acc + static_cast<float>(c) * f;
    }
}

template <typename R>
__device__ __forceinline__ R ld(const R* __restrict__ p, long long off) {
    return __ldg(p + off);
}

// Ordered sum c0*f(o0) + c1*f(o1) + ... with every product and sum rounded.
template <typename R, int N>
__device__ __forceinline__ R ordered(const R* __restrict__ p, long long s, const int (&off)[N],
                                     const double (&c)[N]) {
    R acc = Num<R>::mul(static_cast<R>(c[0]), ld(p, off[0] * s));
#pragma unroll
    for (int t = 1; t < N; ++t) acc = mac(acc, c[t], ld(p, off[t] * s));
    return acc;
}

// ---------------------------------------------------------------------------
// one-sided closures (JAX_BSSN/evolution/derivatives.py:99-160, 398-458, 511-596)
// `p` points at the sample where the closure is evaluated; `first` is the
// offset (in samples along the axis) of the first closure node.
// ---------------------------------------------------------------------------
template <typename R, int N>
__device__ __forceinline__ R closure(const R* __restrict__ p, long long s, int first, const double (&c)[N]) {
    if constexpr (std::is_same<R, float>::value) {
        // the rows' coefficients sum to zero and include the centre sample
        const float f0 = ld(p, 0);
        float acc = 0.0f;
#pragma unroll
        for (int t = 0; t < N; ++t)
            if (first + t != 0) acc += static_cast<float>(c[t]) * (ld(p, (long long)(first + t) * s) - f0);
        return acc;
    } else {
        R acc = Num<R>::mul(static_cast<R>(c[0]), ld(p, (long long)first * s));
#pragma unroll
        for (int t = 1; t < N; ++t) acc = mac(acc, c[t], ld(p, (long long)(first + t) * s));
        return acc;
    }
}

// Stride of axis d in samples.  z runs fastest in every layout (st[2] = 1).
// The float kernels, bound by instruction issue, take the constant for z, so
// a stencil along z addresses its taps with immediate offsets (7-8% of the
// FP32 step); the FP64 kernels read it from the geometry, since the constant
// raised k_rhs_curv's registers from 168 to 198 and slowed the FP64 step 7%.
template <typename R>
__device__ __forceinline__ long long axis_stride(const Geo& G, int d) {
    if constexpr (std::is_same<R, float>::value) return d == 2 ? 1LL : G.st[d];
    else return G.st[d];
}

// Which closure row (0, 1, 2) applies at padded index i, or -1.  The upper
// face is checked first because the reference applies it last (it wins when
// the two faces overlap on a tiny axis).
// Closed = false instantiates a stencil for samples at least kClosureRows
// from every closed face (the interior of a box): no face-row checks at all.
constexpr int kClosureRows = 3;

template <bool Closed = true>
__device__ __forceinline__ int right_row(const Axis& a, int i, int width) {
    if constexpr (!Closed) return -1;
    int r = a.end - 1 - i;
    return (a.rbc && r >= 0 && r < width) ? r : -1;
}
template <bool Closed = true>
__device__ __forceinline__ int left_row(const Axis& a, int i, int width) {
    if constexpr (!Closed) return -1;
    int r = i - a.start;
    return (a.lbc && r >= 0 && r < width) ? r : -1;
}

// ---------------------------------------------------------------------------
// centred first derivative
// ---------------------------------------------------------------------------
template <typename R>
__device__ __forceinline__ R d1_interior(const R* __restrict__ p, long long s, const Axis& a, const Geo& G,
                                         bool mad) {
    const R c1 = ld(p, s) - ld(p, -s);
    const R c2 = ld(p, 2 * s) - ld(p, -2 * s);
    const R d4 = c1 * BSSN_CO(R, G, d1a) + c2 * BSSN_CO(R, G, d1b);
    if (!mad) return d4;
    const R c3 = ld(p, 3 * s) - ld(p, -3 * s);
    const R d6 = (static_cast<R>(3.0 / 4.0) * c1 - static_cast<R>(3.0 / 20.0) * c2 + static_cast<R>(1.0 / 60.0) * c3)
                 * BSSN_CO(R, G, inv_dx);
    return BSSN_AQ(R, a) * d4 + BSSN_AOMQ(R, a) * d6;
}

template <typename R, bool Closed = true>
__device__ __forceinline__ R d1_closed(const R* __restrict__ p, long long s, const Axis& a, int i, const Geo& G,
                                       bool mad) {
    constexpr double L0[5] = {-25.0 / 12.0, 4.0, -3.0, 4.0 / 3.0, -1.0 / 4.0};
    constexpr double L1[5] = {-1.0 / 4.0, -5.0 / 6.0, 3.0 / 2.0, -1.0 / 2.0, 1.0 / 12.0};
    constexpr double R0[5] = {1.0 / 4.0, -4.0 / 3.0, 3.0, -4.0, 25.0 / 12.0};
    constexpr double R1[5] = {-1.0 / 12.0, 1.0 / 2.0, -3.0 / 2.0, 5.0 / 6.0, 1.0 / 4.0};
    const R inv_dx = BSSN_CO(R, G, inv_dx);
    int r = right_row<Closed>(a, i, 2);
    if (r == 0) return closure(p, s, -4, R0) * inv_dx;
    if (r == 1) return closure(p, s, -3, R1) * inv_dx;
    r = left_row<Closed>(a, i, 2);
    if (r == 0) return closure(p, s, 0, L0) * inv_dx;
    if (r == 1) return closure(p, s, -1, L1) * inv_dx;
    return d1_interior(p, s, a, G, mad);
}

// D1 along axis d at padded index i (reduced axes give zero).
template <typename R, bool Closed = true>
__device__ __forceinline__ R D1(const R* __restrict__ p, const Geo& G, int d, int i) {
    const Axis& a = G.ax[d];
    if (a.reduced) return R(0);
    return d1_closed<R, Closed>(p, axis_stride<R>(G, d), a, i, G, a.mad != 0);
}

// ---------------------------------------------------------------------------
// pure second derivative
// ---------------------------------------------------------------------------
// Interior numerators of a field without a constant background (zero far
// value: At, K, Gt, beta, the off-diagonal gt, and every field of the FP32
// form, which stores perturbations).  Their rounding is relative to the
// field's own scale rather than to an O(1) offset, so the reference's term
// order does not have to be kept: the terms are grouped into symmetric pairs
// and fused multiply-adds.  Template argument Exact = false selects these.
// Float: second differences (f(k) - f(0)) + (f(-k) - f(0)) of the pairs.
template <typename R>
__device__ __forceinline__ R second_difference(const R* __restrict__ p, long long s, int k, R f0) {
    return (ld(p, k * s) - f0) + (ld(p, -k * s) - f0);
}
template <typename R>
__device__ __forceinline__ R d2_num_pairs(const R* __restrict__ p, long long s) {
    if constexpr (std::is_same<R, float>::value) {
        const float f0 = ld(p, 0);
        return 16.0f * second_difference(p, s, 1, f0) - second_difference(p, s, 2, f0);
    } else {
        const R p1 = ld(p, s) + ld(p, -s);
        const R p2 = ld(p, 2 * s) + ld(p, -2 * s);
        return (R(16) * p1 - p2) + R(-30) * ld(p, 0);
    }
}
template <typename R>
__device__ __forceinline__ R ko_num_pairs(const R* __restrict__ p, long long s) {
    if constexpr (std::is_same<R, float>::value) {
        const float f0 = ld(p, 0);
        return (second_difference(p, s, 3, f0) - 6.0f * second_difference(p, s, 2, f0))
               + 15.0f * second_difference(p, s, 1, f0);
    } else {
        const R p1 = ld(p, s) + ld(p, -s);
        const R p2 = ld(p, 2 * s) + ld(p, -2 * s);
        const R p3 = ld(p, 3 * s) + ld(p, -3 * s);
        return ((p3 + R(-6) * p2) + R(15) * p1) + R(-20) * ld(p, 0);
    }
}
// Sixth-order D2 numerator (MAD blend) in symmetric pairs.
template <typename R>
__device__ __forceinline__ R d2_6_num_pairs(const R* __restrict__ p, long long s) {
    if constexpr (std::is_same<R, float>::value) {
        const float f0 = ld(p, 0);
        return (float(1.0 / 90.0) * second_difference(p, s, 3, f0) + float(-3.0 / 20.0) * second_difference(p, s, 2, f0))
               + float(3.0 / 2.0) * second_difference(p, s, 1, f0);
    } else {
        const R p1 = ld(p, s) + ld(p, -s);
        const R p2 = ld(p, 2 * s) + ld(p, -2 * s);
        const R p3 = ld(p, 3 * s) + ld(p, -3 * s);
        return ((R(1.0 / 90.0) * p3 + R(-3.0 / 20.0) * p2) + R(3.0 / 2.0) * p1) + R(-49.0 / 18.0) * ld(p, 0);
    }
}
// Any numerator as a fused multiply-add chain.
template <typename R, int N>
__device__ __forceinline__ R fused(const R* __restrict__ p, long long s, const int (&off)[N], const double (&c)[N]) {
    R acc = static_cast<R>(c[0]) * ld(p, off[0] * s);
#pragma unroll
    for (int t = 1; t < N; ++t) acc = acc + static_cast<R>(c[t]) * ld(p, off[t] * s);
    return acc;
}
template <typename R>
__device__ __forceinline__ R up1_num_fused(const R* __restrict__ p, long long s, R c) {
    if (c > R(0))
        return (((R(-3) * ld(p, -s) + R(-10) * ld(p, 0)) + R(18) * ld(p, s)) + R(-6) * ld(p, 2 * s)) + ld(p, 3 * s);
    return (((-ld(p, -3 * s) + R(6) * ld(p, -2 * s)) + R(-18) * ld(p, -s)) + R(10) * ld(p, 0)) + R(3) * ld(p, s);
}

template <typename R, bool Closed = true, bool Exact = true>
__device__ __forceinline__ R D2(const R* __restrict__ p, const Geo& G, int d, int i) {
    const Axis& a = G.ax[d];
    if (a.reduced) return R(0);
    const long long s = axis_stride<R>(G, d);
    constexpr double L0[6] = {15.0 / 4.0, -77.0 / 6.0, 107.0 / 6.0, -13.0, 61.0 / 12.0, -5.0 / 6.0};
    constexpr double L1[6] = {5.0 / 6.0, -5.0 / 4.0, -1.0 / 3.0, 7.0 / 6.0, -1.0 / 2.0, 1.0 / 12.0};
    constexpr double R0[6] = {-5.0 / 6.0, 61.0 / 12.0, -13.0, 107.0 / 6.0, -77.0 / 6.0, 15.0 / 4.0};
    constexpr double R1[6] = {1.0 / 12.0, -1.0 / 2.0, 7.0 / 6.0, -1.0 / 3.0, -5.0 / 4.0, 5.0 / 6.0};
    const R inv_dx2 = BSSN_CO(R, G, inv_dx2);
    int r = right_row<Closed>(a, i, 2);
    if (r == 0) return closure(p, s, -5, R0) * inv_dx2;
    if (r == 1) return closure(p, s, -4, R1) * inv_dx2;
    r = left_row<Closed>(a, i, 2);
    if (r == 0) return closure(p, s, 0, L0) * inv_dx2;
    if (r == 1) return closure(p, s, -1, L1) * inv_dx2;
    constexpr int o4[5] = {2, 1, 0, -1, -2};
    constexpr double c4[5] = {-1.0, 16.0, -30.0, 16.0, -1.0};
    const R d4 = (Exact ? ordered(p, s, o4, c4) : d2_num_pairs(p, s)) * BSSN_CO(R, G, inv_12dx2);
    if (!a.mad) return d4;
    constexpr int o6[7] = {3, 2, 1, 0, -1, -2, -3};
    constexpr double c6[7] = {1.0 / 90.0, -3.0 / 20.0, 3.0 / 2.0, -49.0 / 18.0,
                              3.0 / 2.0, -3.0 / 20.0, 1.0 / 90.0};
    const R d6 = (Exact ? ordered(p, s, o6, c6) : d2_6_num_pairs(p, s)) * inv_dx2;
    return BSSN_AQ(R, a) * d4 + BSSN_AOMQ(R, a) * d6;
}

// ---------------------------------------------------------------------------
// undivided sixth difference along one axis (one KO numerator; the factor
// nu/64 * h^5/dx^6 is applied once to the sum over axes)
// ---------------------------------------------------------------------------
template <typename R, bool Closed = true, bool Exact = true>
__device__ __forceinline__ R KO1(const R* __restrict__ p, const Geo& G, int d, int i) {
    const Axis& a = G.ax[d];
    if (a.reduced) return R(0);
    const long long s = axis_stride<R>(G, d);
    constexpr double L0[8] = {4.0, -27.0, 78.0, -125.0, 120.0, -69.0, 22.0, -3.0};
    constexpr double L1[8] = {3.0, -20.0, 57.0, -90.0, 85.0, -48.0, 15.0, -2.0};
    constexpr double L2[8] = {2.0, -13.0, 36.0, -55.0, 50.0, -27.0, 8.0, -1.0};
    constexpr double R0[8] = {-3.0, 22.0, -69.0, 120.0, -125.0, 78.0, -27.0, 4.0};
    constexpr double R1[8] = {-2.0, 15.0, -48.0, 85.0, -90.0, 57.0, -20.0, 3.0};
    constexpr double R2[8] = {-1.0, 8.0, -27.0, 50.0, -55.0, 36.0, -13.0, 2.0};
    R num;
    int r = right_row<Closed>(a, i, 3);
    if (r == 0) num = closure(p, s, -7, R0);
    else if (r == 1) num = closure(p, s, -6, R1);
    else if (r == 2) num = closure(p, s, -5, R2);
    else {
        r = left_row<Closed>(a, i, 3);
        if (r == 0) num = closure(p, s, 0, L0);
        else if (r == 1) num = closure(p, s, -1, L1);
        else if (r == 2) num = closure(p, s, -2, L2);
        else if (Exact) {
            constexpr int o[7] = {3, 2, 1, 0, -1, -2, -3};
            constexpr double c[7] = {1.0, -6.0, 15.0, -20.0, 15.0, -6.0, 1.0};
            num = ordered(p, s, o, c);
        } else {
            num = ko_num_pairs(p, s);
        }
    }
    return num;
}

// nu/64 * sum_d h^5 D6_d f  (JAX_BSSN/evolution/spatial_derivatives.py:81-92);
// every axis shares h^5/dx^6, so it is applied with nu/64 to the summed
// numerators.
template <typename R, bool Closed = true, bool Exact = true>
__device__ __forceinline__ R KO(const R* __restrict__ p, const Geo& G, const int (&ix)[3]) {
    if constexpr (!Closed && !Exact) {
        R t[3];
#pragma unroll
        for (int d = 0; d < 3; ++d) t[d] = G.ax[d].reduced ? R(0) : ko_num_pairs(p, axis_stride<R>(G, d));
        return BSSN_CO(R, G, ko_scale) * ((t[0] + t[1]) + t[2]);
    }
    const R t = KO1<R, Closed, Exact>(p, G, 0, ix[0]) + KO1<R, Closed, Exact>(p, G, 1, ix[1]);
    return BSSN_CO(R, G, ko_scale) * (t + KO1<R, Closed, Exact>(p, G, 2, ix[2]));
}

// ---------------------------------------------------------------------------
// upwind first derivative selected by the sign of the RHS coefficient c
// ---------------------------------------------------------------------------
template <typename R, bool Closed = true, bool Exact = true>
__device__ __forceinline__ R UP1(const R* __restrict__ p, const Geo& G, int d, int i, R c) {
    const Axis& a = G.ax[d];
    if (a.reduced) return R(0);
    const long long s = axis_stride<R>(G, d);
    const bool physical = Closed && (a.lbc || a.rbc);
    if (physical) {
        // Outer three owned samples at a Sommerfeld face use the closed centred D4
        // (JAX_BSSN/evolution/derivatives.py:296-331).
        const int w = (a.P < 3) ? a.P : 3;
        int lo_r = a.end - w;
        if (lo_r < 0) lo_r = 0;
        if (lo_r > a.P - w) lo_r = a.P - w;
        int lo_l = a.start;
        if (lo_l < 0) lo_l = 0;
        if (lo_l > a.P - w) lo_l = a.P - w;
        if ((a.rbc && i >= lo_r && i < lo_r + w) || (a.lbc && i >= lo_l && i < lo_l + w))
            return d1_closed(p, s, a, i, G, false);
    }
    const R inv_12dx = BSSN_CO(R, G, inv_12dx);
    if (c > R(0)) {
        constexpr int o[5] = {-1, 0, 1, 2, 3};
        constexpr double k[5] = {-3.0, -10.0, 18.0, -6.0, 1.0};
        const R d4 = (Exact ? ordered(p, s, o, k) : up1_num_fused(p, s, c)) * inv_12dx;
        if (!a.mad) return d4;
        constexpr int o6[7] = {-2, -1, 0, 1, 2, 3, 4};
        constexpr double k6[7] = {2.0, -24.0, -35.0, 80.0, -30.0, 8.0, -1.0};
        const R n6 = Exact ? ordered(p, s, o6, k6) : fused(p, s, o6, k6);
        return BSSN_AQ(R, a) * d4 + BSSN_AOMQ(R, a) * (n6 * BSSN_CO(R, G, inv_60dx));
    }
    if (c < R(0)) {
        constexpr int o[5] = {-3, -2, -1, 0, 1};
        constexpr double k[5] = {-1.0, 6.0, -18.0, 10.0, 3.0};
        const R d4 = (Exact ? ordered(p, s, o, k) : up1_num_fused(p, s, c)) * inv_12dx;
        if (!a.mad) return d4;
        constexpr int o6[7] = {-4, -3, -2, -1, 0, 1, 2};
        constexpr double k6[7] = {1.0, -8.0, 30.0, -80.0, 35.0, 24.0, -2.0};
        const R n6 = Exact ? ordered(p, s, o6, k6) : fused(p, s, o6, k6);
        return BSSN_AQ(R, a) * d4 + BSSN_AOMQ(R, a) * (n6 * BSSN_CO(R, G, inv_60dx));
    }
    // zero coefficient (or NaN): centred (JAX_BSSN/evolution/derivatives.py:238-241,272-276)
    return d1_interior(p, s, a, G, a.mad != 0);
}

// Interior D4 upwind numerator in units of 1/(12 dx), the side picked by the
// sign of c.  A zero or NaN coefficient takes the second side: the caller
// multiplies by c/(12 dx), which gives the zero or NaN that UP1's centred
// value times c gives.
template <typename R>
__device__ __forceinline__ R up1_num(const R* __restrict__ p, long long s, R c) {
    if (c > R(0)) {
        constexpr int o[5] = {-1, 0, 1, 2, 3};
        constexpr double k[5] = {-3.0, -10.0, 18.0, -6.0, 1.0};
        return ordered(p, s, o, k);
    }
    constexpr int o[5] = {-3, -2, -1, 0, 1};
    constexpr double k[5] = {-1.0, 6.0, -18.0, 10.0, 3.0};
    return ordered(p, s, o, k);
}

// Shift over 12 dx: the factor of the interior upwind numerators.
template <typename R>
__device__ __forceinline__ void shift_over_12dx(const Geo& G, const R (&beta)[3], R (&bs)[3]) {
#pragma unroll
    for (int d = 0; d < 3; ++d) bs[d] = beta[d] * BSSN_CO(R, G, inv_12dx);
}

// beta^d d_d f summed over d (JAX_BSSN/bssn/shift_and_lapse.py:43-63).  bs is
// beta/(12 dx): closure-free D4 axes multiply it into the bare numerator.
template <typename R, bool Closed = true, bool Exact = true>
__device__ __forceinline__ R ADV(const R* __restrict__ p, const Geo& G, const int (&ix)[3], const R (&beta)[3],
                                 const R (&bs)[3]) {
    R t[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        const Axis& a = G.ax[d];
        if (!Closed && !a.mad)
            t[d] = a.reduced ? R(0)
                             : bs[d] * (Exact ? up1_num(p, axis_stride<R>(G, d), beta[d]) : up1_num_fused(p, axis_stride<R>(G, d), beta[d]));
        else
            t[d] = beta[d] * UP1<R, Closed, Exact>(p, G, d, ix[d], beta[d]);
    }
    return (t[0] + t[1]) + t[2];
}

}  // namespace bssn
