// Cartoon reductions on GB300: axisymmetric (z axis) and spherical.
//
// The evolved state is compact: (Nrho+4, 1, Nz) for axisymmetry, (Nr+4, 1, 1)
// for spherical symmetry, with four parity ghosts at negative x.  Before every
// RHS the positive half-plane (half-line) is interpolated onto a Cartesian
// support -- nine y planes (9 x 9 y-z lines) -- and rotated into the Cartesian
// frame; the unchanged Cartesian RHS is then evaluated on the centre plane
// (centre line) only.  Every stencil there reaches at most four samples in y
// and z, and the support is nine samples wide, so the centre values never see
// the support's periodic wrap: the result equals the reference's RHS on the
// whole support restricted to that plane.
//
// Algorithms (uwplasma/JAX_BSSN):
//   parity ghosts                  JAX_BSSN/cartoon/axisymmetry/reconstruction.py:34-143,
//                                  JAX_BSSN/cartoon/symmetry.py:55-71
//   1/r outer buffer, geometry     reconstruction.py:146-178
//   six-node Lagrange (NaN out)    JAX_BSSN/cartoon/interpolation.py:9-87
//   rotation                       reconstruction.py:206-289
//   centre-plane projection, RK4   reconstruction.py:292-300, axisymmetry/evolution.py:18-65
//   spherical subspace, support    JAX_BSSN/cartoon/spherical_symmetry/reconstruction.py:147-398
//   spherical RK4                  JAX_BSSN/cartoon/spherical_symmetry/evolution.py:17-72
// Interpolation sums and rotation contractions use round-to-nearest
// intrinsics in the reference's order (nodes left to right; tensor
// contraction a-major, b-minor over (L_ia L_jb) T_ab).
#include <cmath>
#include <cstring>

#include "../../include/bssn_gb300.h"
#include "bssn_driver.h"
#include "bssn_fields.cuh"
#include "bssn_kernels.h"
#include "bssn_profile.h"

namespace bssn {
namespace {

constexpr int kCG = 4;        // parity ghosts
constexpr int kSup = 9;       // support width
constexpr int kCenter = 4;    // centre index of the support
constexpr int kThr = 256;
inline unsigned blocks(long long n) { return (unsigned)((n + kThr - 1) / kThr); }

#define RN_ADD __dadd_rn
#define RN_MUL __dmul_rn
#define RN_DIV __ddiv_rn

// reflection parity of a component: axisymmetric (-1,-1,+1), spherical (-1,+1,+1)
__host__ __device__ inline double comp_parity(int c, const double (&p)[3]) {
    if (c <= GZZ || (c >= AXX && c <= AZZ)) {
        const int s = c <= GZZ ? c : c - AXX;
        const int i = s < 3 ? 0 : (s < 5 ? 1 : 2);
        const int j = s < 3 ? s : (s < 5 ? s - 2 : 2);
        return p[i] * p[j];
    }
    if (c >= GTX && c <= GTZ) return p[c - GTX];
    if (c >= BX && c <= BZ) return p[c - BX];
    return 1.0;
}

__host__ __device__ inline double comp_asymptote(int c) {
    return (c == GXX || c == GYY || c == GZZ || c == CW || c == CALPHA) ? 1.0 : 0.0;
}

struct Compact {
    int nx, nz;        // compact extents (nx includes the four ghosts)
    long long cs;      // nx * nz
};

// ---------------------------------------------------------------------------
// parity ghosts: x in [0, 4) from x' = 7 - x on the positive side
// ---------------------------------------------------------------------------
__global__ void k_ghosts(double* __restrict__ u, Compact C, double p0, double p1, double p2) {
    const long long n = (long long)kCG * C.nz * NCOMP;
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    const int c = (int)(t / ((long long)kCG * C.nz));
    const long long r = t - (long long)c * kCG * C.nz;
    const int x = (int)(r / C.nz);
    const int z = (int)(r - (long long)x * C.nz);
    const double p[3] = {p0, p1, p2};
    double* f = u + (long long)c * C.cs;
    f[(long long)x * C.nz + z] = comp_parity(c, p) * f[(long long)(2 * kCG - 1 - x) * C.nz + z];
}

// ---------------------------------------------------------------------------
// six-node weights of the clipped non-periodic stencil (interpolation.py:9-57)
// ---------------------------------------------------------------------------
__device__ inline bool lagrange_nodes(double q, int size, int& start, double (&w)[6]) {
    const int base = (int)floor(q);
    start = base - 2;
    if (start < 0) start = 0;
    if (start > size - 6) start = size - 6;
#pragma unroll
    for (int k = 0; k < 6; ++k) {
        double c = 1.0;
#pragma unroll
        for (int m = 0; m < 6; ++m) {
            if (m == k) continue;
            c = RN_MUL(c, RN_DIV(RN_ADD(q, -(double)(start + m)), (double)((start + k) - (start + m))));
        }
        w[k] = c;
    }
    return q >= 0.0 && q <= (double)(size - 1);
}

// ---------------------------------------------------------------------------
// axisymmetric support (reconstruction.py:146-289)
// ---------------------------------------------------------------------------
struct AxiGeom {
    double dx, zmin;
};

// Write the reconstructed support: point (x, j, z) -> dst at (ox+x, oy+j, oz+z)
// of a block with strides (sx, sy, 1) and component stride dcs.  One block per
// (x, plane pair) and a range of z.  The planes j and 8 - j (y and -y) share
// rho, hence the node window, the six weights and every interpolated profile
// value, and their rotations differ only in the sign of sin(phi): each pair is
// interpolated once and rotated twice.  The window, weights and rotation are
// computed once per block into shared memory; the threads then gather along
// z (coalesced) and rotate.
constexpr int kAxiThreads = 128;
constexpr int kAxiPairs = kCenter + 1;   // planes (j, 8 - j) for j = 0..3, and the centre plane

// Node window, six weights and rotation of one (x, plane pair) column.  They
// depend on the geometry only, so a stepping driver computes the table once
// and every reconstruction of the step reads it (the alternative, thread 0 of
// every block computing its column's chain of FP64 divisions while the block
// waits, dominates the float reconstruction).
struct AxiCol {
    double w[6];
    double cs, sn;
    int start, valid;
};

__device__ __forceinline__ void axi_column(int x, int j, const Compact& C, const AxiGeom& A, AxiCol& out) {
    const double X = RN_MUL((double)x - 3.5, A.dx);
    const double Y = RN_MUL((double)j - 4.0, A.dx);
    const double rho = __dsqrt_rn(RN_ADD(RN_MUL(X, X), RN_MUL(Y, Y)));
    const double q = RN_ADD(RN_ADD(RN_DIV(rho, A.dx), 4.0), -0.5);
    int start;
    double w[6];
    out.valid = lagrange_nodes(q, C.nx + 3, start, w) ? 1 : 0;
    out.start = start;
    for (int k = 0; k < 6; ++k) out.w[k] = w[k];
    // rotation by phi about z: L = [[c,-s,0],[s,c,0],[0,0,1]]
    out.cs = rho <= 0.0 ? 1.0 : RN_DIV(X, rho);
    out.sn = rho <= 0.0 ? 0.0 : RN_DIV(Y, rho);
}

__global__ void k_axi_columns(Compact C, AxiGeom A, AxiCol* __restrict__ T) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= C.nx * kAxiPairs) return;
    axi_column(t / kAxiPairs, t - (t / kAxiPairs) * kAxiPairs, C, A, T[t]);
}

// mode 0: every plane.  mode 1 (the FP32 form, whose support is
// reconstructed in float): W alone, on the off-centre plane pairs.  mode 2:
// every component on the off-centre pairs.  In modes 1 and 2 the centre plane
// comes from k_copy_centre.  T: the column table, or null (each block then
// computes its column).
__global__ void __launch_bounds__(kAxiThreads) k_axi_reconstruct(const double* __restrict__ u, Compact C, AxiGeom A,
                                                                 double* __restrict__ dst, long long dcs, long long sx,
                                                                 long long sy, int ox, int oy, int oz, int mode,
                                                                 const AxiCol* __restrict__ T) {
    __shared__ double s_w[6];
    __shared__ double s_cs, s_sn;
    __shared__ int s_start, s_valid;
    const int col = blockIdx.x;            // x * kAxiPairs + j
    const int x = col / kAxiPairs, j = col - (col / kAxiPairs) * kAxiPairs;
    if (mode != 0 && j == kCenter) return;    // block-uniform
    if (threadIdx.x == 0) {
        AxiCol K;
        if (T) K = T[col];
        else axi_column(x, j, C, A, K);
        s_valid = K.valid;
        s_start = K.start;
        for (int k = 0; k < 6; ++k) s_w[k] = K.w[k];
        s_cs = K.cs;
        s_sn = K.sn;
    }
    __syncthreads();
    const int z = blockIdx.y * kAxiThreads + threadIdx.x;
    if (z >= C.nz) return;
    const int start = s_start;
    const bool valid = s_valid != 0;
    double w[6];
#pragma unroll
    for (int k = 0; k < 6; ++k) w[k] = s_w[k];
    // 1/r continuation ratios of the three buffer samples at this z (reconstruction.py:146-167)
    double ratio[3] = {0.0, 0.0, 0.0};
    if (start + 5 >= C.nx) {
        const double rho_edge = RN_MUL((double)(C.nx - kCG) - 0.5, A.dx);
        const double zc = RN_ADD(A.zmin, RN_MUL(A.dx, (double)z));
        const double zz = RN_MUL(zc, zc);
        const double r_edge = __dsqrt_rn(RN_ADD(RN_MUL(rho_edge, rho_edge), zz));
#pragma unroll
        for (int b = 0; b < 3; ++b) {
            const double rho_b = RN_ADD(rho_edge, RN_MUL(A.dx, (double)(b + 1)));
            ratio[b] = RN_DIV(r_edge, __dsqrt_rn(RN_ADD(RN_MUL(rho_b, rho_b), zz)));
        }
    }
    const double par3[3] = {-1.0, -1.0, 1.0};
    const double nan = __longlong_as_double(0x7ff8000000000000LL);
    const bool only_w = mode == 1;
    // six-node sum of every component (reflected plane, then the buffer)
    double val[NCOMP];
#pragma unroll
    for (int c = 0; c < NCOMP; ++c) {
        if (only_w && c != CW) continue;
        const double* f = u + (long long)c * C.cs;
        const double par = comp_parity(c, par3);
        const double asym = comp_asymptote(c);
        double acc = 0.0;
#pragma unroll
        for (int k = 0; k < 6; ++k) {
            const int src = start + k;
            double v;
            if (src < kCG) v = par * f[(long long)(2 * kCG - 1 - src) * C.nz + z];
            else if (src < C.nx) v = f[(long long)src * C.nz + z];
            else v = RN_ADD(asym, RN_MUL(RN_ADD(f[(long long)(C.nx - 1) * C.nz + z], -asym), ratio[src - C.nx]));
            acc = k == 0 ? RN_MUL(v, w[0]) : RN_ADD(acc, RN_MUL(v, w[k]));
        }
        val[c] = valid ? acc : nan;
    }
    // L = R_z(phi) = [[c,-s,0],[s,c,0],[0,0,1]].  Its four literal zeros
    // (L_i2, L_2a for i, a < 2) only add (+-0) T terms to the reference's
    // sums, so they are skipped: the remaining terms keep the reference's
    // order (vector: j ascending; tensor: a-major, b-minor over (L_ia L_jb) T_ab),
    // and the result differs at most in the sign of a zero (or, for a
    // non-finite input, in not turning 0 * inf into NaN).  The mirrored plane
    // has y -> -y, so sin(phi) -> -sin(phi) exactly.
    auto rotate_write = [&](int plane, double sn) {
        const double L[3][3] = {{s_cs, -sn, 0.0}, {sn, s_cs, 0.0}, {0.0, 0.0, 1.0}};
        const long long d = (long long)(ox + x) * sx + (long long)(oy + plane) * sy + (oz + z);
        dst[(long long)CW * dcs + d] = val[CW];
        if (only_w) return;
        dst[(long long)CK * dcs + d] = val[CK];
        dst[(long long)CALPHA * dcs + d] = val[CALPHA];
#pragma unroll
        for (int base = 0; base < 2; ++base) {
            const int off = base == 0 ? GTX : BX;
#pragma unroll
            for (int i = 0; i < 2; ++i)
                dst[(long long)(off + i) * dcs + d] = RN_ADD(RN_MUL(L[i][0], val[off]), RN_MUL(L[i][1], val[off + 1]));
            dst[(long long)(off + 2) * dcs + d] = val[off + 2];
        }
#pragma unroll
        for (int base = 0; base < 2; ++base) {
            const int off = base == 0 ? GXX : AXX;
#pragma unroll
            for (int i = 0; i < 3; ++i)
#pragma unroll
                for (int jj = i; jj < 3; ++jj) {
                    double acc = 0.0;
                    bool first = true;
#pragma unroll
                    for (int ab = 0; ab < 9; ++ab) {
                        const int a2 = ab / 3, b2 = ab % 3;
                        if ((i == 2) != (a2 == 2) || (jj == 2) != (b2 == 2)) continue;   // literal zero of L
                        const double term = RN_MUL(RN_MUL(L[i][a2], L[jj][b2]), val[off + sym(a2, b2)]);
                        acc = first ? term : RN_ADD(acc, term);
                        first = false;
                    }
                    dst[(long long)(off + sym(i, jj)) * dcs + d] = acc;
                }
        }
    };
    rotate_write(j, s_sn);
    if (j != kCenter) rotate_write(kSup - 1 - j, -s_sn);
}

// ---------------------------------------------------------------------------
// FP32 form: the axisymmetric support in float.  The FP32 RHS reads float
// perturbations of the support about fixed backgrounds (1 for the metric
// diagonal, W and alpha; the value at the first positive sample of z row 0
// for the shift and K; 0 else).  Interpolation weights sum to one, so the
// perturbation of an interpolated profile is the interpolated perturbation;
// the reflected ghosts and the 1/r buffer add the background terms their
// parity and asymptote produce; the rotation preserves the identity metric,
// and a uniform shift background b gains R b - b.  So the support is
// reconstructed from float perturbations of the compact state, in float, and
// only the centre plane (full values at the points) and W (1/W of the
// derived fields) stay FP64 (k_axi_reconstruct with w_only).
// ---------------------------------------------------------------------------
__device__ __forceinline__ double axi_background(const double* __restrict__ u, const Compact& C, int c) {
    if (comp_asymptote(c) != 0.0) return 1.0;
    if (c == BX || c == BY || c == BZ || c == CK) return u[(long long)c * C.cs + (long long)kCG * C.nz];
    return 0.0;
}

// The support's centre plane is the compact state itself: there every column
// sits on a node (weights 0, 0, 1, 0, 0, 0) and the rotation is the identity
// (x >= 4) or by pi (the ghost columns, which hold exactly the parity images
// it produces), so for finite values the reconstruction returns the compact
// samples bit for bit.
__global__ void k_copy_centre(const double* __restrict__ u, Compact C, double* __restrict__ dst, long long dcs,
                              long long sx, long long sy, int ox, int oy, int oz) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= C.cs * NCOMP) return;
    const int c = (int)(t / C.cs);
    const long long r = t - (long long)c * C.cs;
    const int x = (int)(r / C.nz), z = (int)(r - (long long)x * C.nz);
    dst[(long long)c * dcs + (long long)(ox + x) * sx + (long long)(oy + kCenter) * sy + (oz + z)] = u[t];
}

__global__ void k_compact_f32(const double* __restrict__ u, Compact C, float* __restrict__ cf) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= C.cs * NCOMP) return;
    const int c = (int)(t / C.cs);
    cf[t] = static_cast<float>(u[t] - axi_background(u, C, c));
}

// Float-float accumulation of products: s + c carries a sum of products v w
// (w given as a float pair hi + lo) to about 2^-46 of its size, so the
// interpolation and rotation round once, at the final float, like the FP64
// path's final conversion.
struct FF {
    float s = 0.f, c = 0.f;
    __device__ __forceinline__ void add_prod(float v, float whi, float wlo) {
        // _rn intrinsics: no contraction may merge the product into the sums
        const float p = __fmul_rn(v, whi);
        const float pe = fmaf(v, whi, -p);   // exact error of the product
        const float t = __fadd_rn(s, p);
        const float z = __fsub_rn(t, s);
        const float te = __fadd_rn(__fsub_rn(s, __fsub_rn(t, z)), __fsub_rn(p, z));   // TwoSum error
        c += te + pe + v * wlo;
        s = t;
    }
    __device__ __forceinline__ float value() const { return s + c; }
};

// The rotation coefficients L_ia L_jb (tensors) and L_ia (vectors) of one
// plane, as float pairs: index q over the tensor terms that are not literal
// zeros (xx 4, xy 4, xz 2, yy 4, yz 2, zz 1), then the four vector entries.
constexpr int kRotTensorTerms = 17;
constexpr int kRotTerms = kRotTensorTerms + 4;

__device__ void rotation_pairs(double cs, double sn, float* hi, float* lo) {
    const double L[3][3] = {{cs, -sn, 0.0}, {sn, cs, 0.0}, {0.0, 0.0, 1.0}};
    int q = 0;
    for (int i = 0; i < 3; ++i)
        for (int jj = i; jj < 3; ++jj)
            for (int ab = 0; ab < 9; ++ab) {
                const int a2 = ab / 3, b2 = ab % 3;
                if ((i == 2) != (a2 == 2) || (jj == 2) != (b2 == 2)) continue;
                const double v = L[i][a2] * L[jj][b2];
                hi[q] = static_cast<float>(v);
                lo[q] = static_cast<float>(v - (double)hi[q]);
                ++q;
            }
    const double vec[4] = {L[0][0], L[0][1], L[1][0], L[1][1]};
    for (int k = 0; k < 4; ++k, ++q) {
        hi[q] = static_cast<float>(vec[k]);
        lo[q] = static_cast<float>(vec[k] - (double)hi[q]);
    }
}

__global__ void __launch_bounds__(kAxiThreads)
k_axi_reconstruct_f32(const float* __restrict__ cf, const double* __restrict__ u, Compact C, AxiGeom A,
                      float* __restrict__ dst, long long dcs, long long sx, long long sy, int ox, int oy, int oz,
                      const AxiCol* __restrict__ T) {
    __shared__ float s_w[6], s_wlo[6];
    __shared__ float s_cs, s_sn;
    __shared__ int s_start, s_valid;
    __shared__ float s_b[NCOMP], s_par[NCOMP], s_asym[NCOMP];
    __shared__ float s_rhi[2][kRotTerms], s_rlo[2][kRotTerms];   // plane j, mirrored plane
    const int col = blockIdx.x;
    const int x = col / kAxiPairs, j = col - (col / kAxiPairs) * kAxiPairs;
    if (threadIdx.x == 0) {
        AxiCol K;
        if (T) K = T[col];
        else axi_column(x, j, C, A, K);
        s_valid = K.valid;
        s_start = K.start;
        for (int k = 0; k < 6; ++k) {
            s_w[k] = static_cast<float>(K.w[k]);
            s_wlo[k] = static_cast<float>(K.w[k] - (double)s_w[k]);
        }
        s_cs = static_cast<float>(K.cs);
        s_sn = static_cast<float>(K.sn);
        rotation_pairs(K.cs, K.sn, s_rhi[0], s_rlo[0]);
        rotation_pairs(K.cs, -K.sn, s_rhi[1], s_rlo[1]);
    }
    if (threadIdx.x < NCOMP) {
        const double par3[3] = {-1.0, -1.0, 1.0};
        s_b[threadIdx.x] = static_cast<float>(axi_background(u, C, threadIdx.x));
        s_par[threadIdx.x] = static_cast<float>(comp_parity(threadIdx.x, par3));
        s_asym[threadIdx.x] = static_cast<float>(comp_asymptote(threadIdx.x));
    }
    __syncthreads();
    const int z = blockIdx.y * kAxiThreads + threadIdx.x;
    if (z >= C.nz) return;
    const int start = s_start;
    const bool valid = s_valid != 0;
    float w[6], wlo[6];
#pragma unroll
    for (int k = 0; k < 6; ++k) {
        w[k] = s_w[k];
        wlo[k] = s_wlo[k];
    }
    float ratio[3] = {0.f, 0.f, 0.f};
    if (start + 5 >= C.nx) {
        const double rho_edge = RN_MUL((double)(C.nx - kCG) - 0.5, A.dx);
        const double zc = RN_ADD(A.zmin, RN_MUL(A.dx, (double)z));
        const double zz = RN_MUL(zc, zc);
        const double r_edge = __dsqrt_rn(RN_ADD(RN_MUL(rho_edge, rho_edge), zz));
#pragma unroll
        for (int b = 0; b < 3; ++b) {
            const double rho_b = RN_ADD(rho_edge, RN_MUL(A.dx, (double)(b + 1)));
            ratio[b] = static_cast<float>(RN_DIV(r_edge, __dsqrt_rn(RN_ADD(RN_MUL(rho_b, rho_b), zz))));
        }
    }
    const float nan = __int_as_float(0x7fc00000);
    float val[NCOMP];
#pragma unroll
    for (int c = 0; c < NCOMP; ++c) {
        const float* f = cf + (long long)c * C.cs;
        const float par = s_par[c];
        const float b = s_b[c];
        const float asym = s_asym[c];
        FF acc;
#pragma unroll
        for (int k = 0; k < 6; ++k) {
            const int src = start + k;
            float v;
            // perturbations: the reflection par (d + b) - b, the buffer
            // asym + (d_edge + b - asym) r - b
            if (src < kCG) v = fmaf(par, f[(long long)(2 * kCG - 1 - src) * C.nz + z], (par - 1.f) * b);
            else if (src < C.nx) v = f[(long long)src * C.nz + z];
            else {
                const float r = ratio[src - C.nx];
                v = fmaf(f[(long long)(C.nx - 1) * C.nz + z], r, (asym - b) * (1.f - r));
            }
            acc.add_prod(v, w[k], wlo[k]);
        }
        val[c] = valid ? acc.value() : nan;
    }
    auto rotate_write = [&](int plane, int mirror) {
        const float* rh = s_rhi[mirror];
        const float* rl = s_rlo[mirror];
        const float cs = s_cs, sn = mirror ? -s_sn : s_sn;
        const long long d = (long long)(ox + x) * sx + (long long)(oy + plane) * sy + (oz + z);
        dst[(long long)CW * dcs + d] = val[CW];
        dst[(long long)CK * dcs + d] = val[CK];
        dst[(long long)CALPHA * dcs + d] = val[CALPHA];
        // vectors: rows (L_00, L_01), (L_10, L_11) are terms 17-20
#pragma unroll
        for (int base = 0; base < 2; ++base) {
            const int off = base == 0 ? GTX : BX;
#pragma unroll
            for (int i = 0; i < 2; ++i) {
                FF a;
                a.add_prod(val[off], rh[kRotTensorTerms + 2 * i], rl[kRotTensorTerms + 2 * i]);
                a.add_prod(val[off + 1], rh[kRotTensorTerms + 2 * i + 1], rl[kRotTensorTerms + 2 * i + 1]);
                float v = a.value();
                // shift: R (b + d) - b = R d + (R b - b)
                if (base == 1) {
                    const float bx = s_b[BX], by = s_b[BY];
                    v += i == 0 ? (cs - 1.f) * bx - sn * by : sn * bx + (cs - 1.f) * by;
                }
                dst[(long long)(off + i) * dcs + d] = v;
            }
            dst[(long long)(off + 2) * dcs + d] = val[off + 2];
        }
        // metric (background I, preserved) and At (background 0): R T R^T
#pragma unroll
        for (int base = 0; base < 2; ++base) {
            const int off = base == 0 ? GXX : AXX;
            int q = 0;
#pragma unroll
            for (int i = 0; i < 3; ++i)
#pragma unroll
                for (int jj = i; jj < 3; ++jj) {
                    FF a;
#pragma unroll
                    for (int ab = 0; ab < 9; ++ab) {
                        const int a2 = ab / 3, b2 = ab % 3;
                        if ((i == 2) != (a2 == 2) || (jj == 2) != (b2 == 2)) continue;   // literal zero of L
                        a.add_prod(val[off + sym(a2, b2)], rh[q], rl[q]);
                        ++q;
                    }
                    dst[(long long)(off + sym(i, jj)) * dcs + d] = a.value();
                }
        }
    };
    rotate_write(j, 0);
    if (j != kCenter) rotate_write(kSup - 1 - j, 1);
}

// ---------------------------------------------------------------------------
// spherical support (spherical_symmetry/reconstruction.py:192-385)
// ---------------------------------------------------------------------------
__device__ inline double sph_source(const double* __restrict__ f, int nx, int s, double asym, double par,
                                    double dx) {
    if (s < kCG) return par * f[2 * kCG - 1 - s];
    if (s < nx) return f[s];
    const int b = s - nx;
    const double outer = RN_MUL((double)(nx - kCG) - 0.5, dx);
    const double radius = RN_ADD(outer, RN_MUL(dx, (double)(b + 1)));
    return RN_ADD(asym, RN_MUL(RN_ADD(f[nx - 1], -asym), RN_DIV(outer, radius)));
}

__global__ void k_sph_reconstruct(const double* __restrict__ u, int nx, double dx, double* __restrict__ dst,
                                  long long dcs, long long sx, long long sy, int ox, int oy, int oz) {
    const long long n = (long long)nx * kSup * kSup;
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    const int x = (int)(t / (kSup * kSup));
    const int r2 = (int)(t - (long long)x * kSup * kSup);
    const int j = r2 / kSup, k = r2 % kSup;
    const double X = RN_MUL(((double)x - 4.0) + 0.5, dx);
    const double Y = RN_MUL((double)j - 4.0, dx);
    const double Z = RN_MUL((double)k - 4.0, dx);
    const double radius = __dsqrt_rn(RN_ADD(RN_ADD(RN_MUL(X, X), RN_MUL(Y, Y)), RN_MUL(Z, Z)));
    const double q = RN_ADD(RN_ADD(RN_DIV(radius, dx), 4.0), -0.5);
    int start;
    double w[6];
    const bool valid = lagrange_nodes(q, nx + 3, start, w);
    const long long cs = (long long)nx;  // compact component stride (nx x 1 x 1)
    // nine independent profiles: gt_rr, gt_tt, W, At_rr, At_tt, K, Gt_r, alpha, beta_r
    const int src[9] = {GXX, GYY, CW, AXX, AYY, CK, GTX, CALPHA, BX};
    const double asym[9] = {1.0, 1.0, 1.0, 0.0, 0.0, 0.0, 0.0, 1.0, 0.0};
    const double par[9] = {1.0, 1.0, 1.0, 1.0, 1.0, 1.0, -1.0, 1.0, -1.0};
    double prof[9];
#pragma unroll 1
    for (int pi = 0; pi < 9; ++pi) {
        const double* f = u + (long long)src[pi] * cs;
        double acc = RN_MUL(sph_source(f, nx, start, asym[pi], par[pi], dx), w[0]);
#pragma unroll
        for (int kk = 1; kk < 6; ++kk)
            acc = RN_ADD(acc, RN_MUL(sph_source(f, nx, start + kk, asym[pi], par[pi], dx), w[kk]));
        prof[pi] = valid ? acc : __longlong_as_double(0x7ff8000000000000LL);
    }
    // frame: columns radial, azimuthal, polar (reconstruction.py:265-309)
    const double rho = __dsqrt_rn(RN_ADD(RN_MUL(X, X), RN_MUL(Y, Y)));
    const bool off = rho > 0.0;
    const double safe = off ? rho : 1.0;
    const double rs = RN_MUL(radius, safe);
    double L[3][3];
    L[0][0] = RN_DIV(X, radius);
    L[1][0] = RN_DIV(Y, radius);
    L[2][0] = RN_DIV(Z, radius);
    L[0][1] = off ? RN_DIV(-Y, safe) : 0.0;
    L[1][1] = off ? RN_DIV(X, safe) : 1.0;
    L[2][1] = 0.0;
    L[0][2] = off ? RN_DIV(RN_MUL(-X, Z), rs) : RN_DIV(-Z, radius);
    L[1][2] = off ? RN_DIV(RN_MUL(-Y, Z), rs) : 0.0;
    L[2][2] = off ? RN_DIV(rho, radius) : 0.0;
    double out[NCOMP];
    // tensors diag(rr, tt, tt)
#pragma unroll
    for (int base = 0; base < 2; ++base) {
        const int offc = base == 0 ? GXX : AXX;
        const double rr = prof[base == 0 ? 0 : 3], tt = prof[base == 0 ? 1 : 4];
        const double T[3][3] = {{rr, 0.0, 0.0}, {0.0, tt, 0.0}, {0.0, 0.0, tt}};
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int jj = i; jj < 3; ++jj) {
                double acc = RN_MUL(RN_MUL(L[i][0], L[jj][0]), T[0][0]);
#pragma unroll
                for (int ab = 1; ab < 9; ++ab) {
                    const int a = ab / 3, b = ab % 3;
                    acc = RN_ADD(acc, RN_MUL(RN_MUL(L[i][a], L[jj][b]), T[a][b]));
                }
                out[offc + sym(i, jj)] = acc;
            }
    }
    // vectors (v_r, 0, 0)
#pragma unroll
    for (int base = 0; base < 2; ++base) {
        const int offc = base == 0 ? GTX : BX;
        const double vr = prof[base == 0 ? 6 : 8];
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            double acc = RN_MUL(L[i][0], vr);
            acc = RN_ADD(acc, RN_MUL(L[i][1], 0.0));
            acc = RN_ADD(acc, RN_MUL(L[i][2], 0.0));
            out[offc + i] = acc;
        }
    }
    out[CW] = prof[2];
    out[CK] = prof[5];
    out[CALPHA] = prof[7];
    const long long d = (long long)(ox + x) * sx + (long long)(oy + j) * sy + (oz + k);
#pragma unroll
    for (int c = 0; c < NCOMP; ++c) dst[(long long)c * dcs + d] = out[c];
}

// spherical symmetric subspace on the positive half-line (reconstruction.py:147-189)
__global__ void k_sph_symmetry(double* __restrict__ u, int nx) {
    const int x = kCG + (int)(blockIdx.x * blockDim.x + threadIdx.x);
    if (x >= nx) return;
    const long long cs = nx;
    double* v = u + x;
    v[GXY * cs] = 0.0; v[GXZ * cs] = 0.0; v[GYZ * cs] = 0.0; v[GZZ * cs] = v[GYY * cs];
    v[AXY * cs] = 0.0; v[AXZ * cs] = 0.0; v[AYZ * cs] = 0.0; v[AZZ * cs] = v[AYY * cs];
    v[GTY * cs] = 0.0; v[GTZ * cs] = 0.0; v[BY * cs] = 0.0; v[BZ * cs] = 0.0;
}

// copy the support's centre plane/line RHS (x in [4, nx)) into the compact layout
__global__ void k_collect(const double* __restrict__ ks, long long scs, long long sx, long long sy, int oy, int oz,
                          double* __restrict__ kc, Compact C) {
    const long long n = (long long)(C.nx - kCG) * C.nz * NCOMP;
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    const long long per = (long long)(C.nx - kCG) * C.nz;
    const int c = (int)(t / per);
    const long long r = t - (long long)c * per;
    const int x = kCG + (int)(r / C.nz);
    const int z = (int)(r - (long long)(x - kCG) * C.nz);
    kc[(long long)c * C.cs + (long long)x * C.nz + z] =
        ks[(long long)c * scs + (long long)(x + 4) * sx + (long long)oy * sy + (oz + z)];
}

// constraint fields of the support's centre plane (box order) -> compact with parity ghosts
__global__ void k_cons_compact(const double* __restrict__ boxv, Compact C, double* __restrict__ out, int axi) {
    const long long per = (long long)C.nx * C.nz;
    const long long n = per * 9;
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    const int f = (int)(t / per);
    const long long r = t - (long long)f * per;
    const int x = (int)(r / C.nz);
    const int z = (int)(r - (long long)x * C.nz);
    // fields: H, M0, M1, M2, det, trA, G0, G1, G2; vectors carry the reflection parity
    const double pa[3] = {-1.0, axi ? -1.0 : 1.0, 1.0};
    const int vec = (f >= 1 && f <= 3) ? f - 1 : ((f >= 6) ? f - 6 : -1);
    const double par = vec >= 0 ? pa[vec] : 1.0;
    const int xs = x < kCG ? 2 * kCG - 1 - x : x;
    const long long boxn = (long long)(C.nx - kCG) * C.nz;
    const double v = boxv[(long long)f * boxn + (long long)(xs - kCG) * C.nz + z];
    out[(long long)f * per + r] = x < kCG ? par * v : v;
}

// ---------------------------------------------------------------------------
// driver
// ---------------------------------------------------------------------------
struct CartoonPlan {
    bool axi;
    Compact C;
    Geo Gs;           // support geometry (padded by 4)
    Box centre;       // compute box on the support
    Geo Gc;           // compact geometry for the stage epilogue
    Box positive;     // positive compact samples
    long long scs;    // support component stride
    bool with_mom;
};

int cartoon_plan(bool axi, const int32_t shape[3], const BssnParams* p, CartoonPlan& P) {
    int st = validate_params(p);
    if (st) return st;
    if (!shape) return fail(BSSN_ERR_INVALID, "shape is null");
    const int nx = shape[0], ny = shape[1], nz = shape[2];
    if (axi) {
        if (ny != 1) return fail(BSSN_ERR_INVALID, "axisymmetric Cartoon state requires a singleton y plane");
        if (nx - kCG < 6) return fail(BSSN_ERR_INVALID, "axisymmetric Cartoon mode requires at least six radial points");
        if (nz < 9) return fail(BSSN_ERR_INVALID, "axisymmetric Cartoon mode requires at least nine z points");
        if (p->bc[0] != 0) return fail(BSSN_ERR_INVALID, "axisymmetric x-left is a parity ghost region");
        if (p->bc[1] != 1) return fail(BSSN_ERR_INVALID, "axisymmetric x-right must use the Sommerfeld boundary");
        if (p->bc[2] != 0 || p->bc[3] != 0)
            return fail(BSSN_ERR_INVALID, "axisymmetric reconstructed y faces must be periodic");
        const bool z_ok = (p->bc[4] == 0 || p->bc[4] == 1) && (p->bc[5] == 0 || p->bc[5] == 1);
        if (!z_ok) return fail(BSSN_ERR_INVALID, "axisymmetric z faces must be periodic or Sommerfeld");
        if (p->mad_q != 1.0) return fail(BSSN_ERR_INVALID, "axisymmetric Cartoon requires mad_q=1");
        // jnp.isclose defaults: |a - e| <= 1e-8 + 1e-5 |e|
        const double ex = -3.5 * p->dx, ey = -4.0 * p->dx;
        if (!(std::fabs(p->xmin[0] - ex) <= 1e-8 + 1e-5 * std::fabs(ex)))
            return fail(BSSN_ERR_INVALID, "axisymmetric Cartoon requires x_min=-3.5*dx");
        if (!(std::fabs(p->xmin[1] - ey) <= 1e-8 + 1e-5 * std::fabs(ey)))
            return fail(BSSN_ERR_INVALID, "axisymmetric Cartoon requires y_min=-4*dx");
    } else {
        if (ny != 1 || nz != 1) return fail(BSSN_ERR_INVALID, "spherical Cartoon state requires an (Nr + 4) x 1 x 1 grid");
        if (nx - kCG < 6) return fail(BSSN_ERR_INVALID, "spherical Cartoon mode requires at least six radial points");
        if (p->bc[0] != 0) return fail(BSSN_ERR_INVALID, "Cartoon x-left is a parity ghost region, not a physical boundary");
        if (p->bc[1] != 1) return fail(BSSN_ERR_INVALID, "Cartoon x-right must use the Sommerfeld boundary");
        for (int f = 2; f < 6; ++f)
            if (p->bc[f] != 0) return fail(BSSN_ERR_INVALID, "Cartoon y/z support faces must be periodic");
        if (p->mad_q != 1.0) return fail(BSSN_ERR_INVALID, "Cartoon reconstruction requires mad_q=1 for its 9 x 9 support");
        const double e[3] = {-3.5 * p->dx, -4.0 * p->dx, -4.0 * p->dx};
        for (int d = 0; d < 3; ++d)
            if (!(std::fabs(p->xmin[d] - e[d]) <= 1e-12 * std::fmax(1.0, std::fabs(e[d]))))
                return fail(BSSN_ERR_INVALID, "Cartoon coordinate minima must be (-3.5dx, -4dx, -4dx)");
    }
    if (p->guard_cells != 0 || p->owned_shape[0] >= 0)
        return fail(BSSN_ERR_INVALID, "Cartoon states are whole compact arrays (no guard description)");
    P.axi = axi;
    P.C.nx = nx;
    P.C.nz = axi ? nz : 1;
    P.C.cs = (long long)nx * P.C.nz;
    const int S[3] = {nx, kSup, axi ? nz : kSup};
    const int org[3] = {4, 4, 4};
    const int Pd[3] = {S[0] + 8, S[1] + 8, S[2] + 8};
    if ((st = make_geo(p, S, org, Pd, P.Gs))) return st;
    P.scs = P.Gs.cs;
    P.centre.lo[0] = 4 + kCG;
    P.centre.n[0] = nx - kCG;
    P.centre.lo[1] = 4 + kCenter;
    P.centre.n[1] = 1;
    P.centre.lo[2] = axi ? 4 : 4 + kCenter;
    P.centre.n[2] = axi ? nz : 1;
    P.centre.count = (long long)P.centre.n[0] * P.centre.n[1] * P.centre.n[2];
    std::memset(&P.Gc, 0, sizeof(P.Gc));
    P.Gc.precision = p->precision;
    P.Gc.st[2] = 1;
    P.Gc.st[1] = P.C.nz;
    P.Gc.st[0] = P.C.nz;
    P.Gc.cs = P.C.cs;
    P.Gc.ninst = 1;
    P.Gc.istride = P.C.cs;
    P.positive.lo[0] = kCG;
    P.positive.n[0] = nx - kCG;
    P.positive.lo[1] = 0;
    P.positive.n[1] = 1;
    P.positive.lo[2] = 0;
    P.positive.n[2] = P.C.nz;
    P.positive.count = (long long)(nx - kCG) * P.C.nz;
    P.with_mom = p->kappa != 0.0;
    return BSSN_OK;
}

// support state + support RHS + RHS work + compact stage, RHS, accumulator
// doubles of the axisymmetric column table
size_t axi_table_values(const CartoonPlan& P) {
    return P.axi ? ((size_t)P.C.nx * kAxiPairs * sizeof(AxiCol) + sizeof(double) - 1) / sizeof(double) : 0;
}

size_t cartoon_step_values(const CartoonPlan& P) {
    return (size_t)(2 * NCOMP + rhs_work_blocks(P.with_mom)) * (size_t)P.scs + 3 * NCOMP * (size_t)P.C.cs +
           axi_table_values(P);
}

// support state + first derivatives + derived blocks + nine constraint blocks of the centre box
size_t cartoon_constraint_values(const CartoonPlan& P) {
    return (size_t)(NCOMP + 3 * NMIX + 24) * (size_t)P.scs + 9 * (size_t)P.centre.count;
}

size_t cartoon_work_values(const CartoonPlan& P) {
    const size_t a = cartoon_step_values(P), b = cartoon_constraint_values(P);
    return a > b ? a : b;
}

cudaError_t reconstruct(const CartoonPlan& P, const BssnParams* p, const double* u, double* us, cudaStream_t s,
                        const AxiCol* T = nullptr) {
    const long long sx = P.Gs.st[0], sy = P.Gs.st[1];
    if (P.axi) {
        const AxiGeom A{p->dx, p->xmin[2]};
        const dim3 grid((unsigned)(P.C.nx * kAxiPairs), (unsigned)((P.C.nz + kAxiThreads - 1) / kAxiThreads));
        if (T) {
            // the stepping driver: centre plane copied (bit-identical for finite
            // values, up to the sign of zeros), the plane pairs reconstructed
            BSSN_LAUNCH(KC_CARTOON, k_copy_centre, blocks(P.C.cs * NCOMP), kThr, s, u, P.C, us, P.scs, sx, sy, 4, 4,
                        4);
            BSSN_LAUNCH(KC_CARTOON, k_axi_reconstruct, grid, kAxiThreads, s, u, P.C, A, us, P.scs, sx, sy, 4, 4, 4, 2,
                        T);
        } else {
            BSSN_LAUNCH(KC_CARTOON, k_axi_reconstruct, grid, kAxiThreads, s, u, P.C, A, us, P.scs, sx, sy, 4, 4, 4, 0,
                        T);
        }
    } else {
        const long long n = (long long)P.C.nx * kSup * kSup;
        BSSN_LAUNCH(KC_CARTOON, k_sph_reconstruct, blocks(n), kThr, s, u, P.C.nx, p->dx, us, P.scs, sx, sy, 4, 4, 4);
    }
    return launch_fill_periodic(us, NCOMP, P.Gs, s);
}

// FP32 form, axisymmetric: FP64 support only on the centre plane and for W,
// float support from float perturbations of the compact state (staged in the
// first-derivative scratch, which the RHS overwrites afterwards).
cudaError_t reconstruct_f32(const CartoonPlan& P, const BssnParams* p, const double* u, double* us, const RhsWork& w,
                            cudaStream_t s, const AxiCol* T) {
    const long long sx = P.Gs.st[0], sy = P.Gs.st[1];
    const AxiGeom A{p->dx, p->xmin[2]};
    const dim3 grid((unsigned)(P.C.nx * kAxiPairs), (unsigned)((P.C.nz + kAxiThreads - 1) / kAxiThreads));
    BSSN_LAUNCH(KC_CARTOON, k_copy_centre, blocks(P.C.cs * NCOMP), kThr, s, u, P.C, us, P.scs, sx, sy, 4, 4, 4);
    BSSN_LAUNCH(KC_CARTOON, k_axi_reconstruct, grid, kAxiThreads, s, u, P.C, A, us, P.scs, sx, sy, 4, 4, 4, 1, T);
    // FP64 values outside the centre box are read for W only
    cudaError_t e = launch_fill_periodic(us + (long long)CW * P.scs, 1, P.Gs, s);
    if (e != cudaSuccess) return e;
    float* cf = w.d1f;
    BSSN_LAUNCH(KC_CONVERT, k_compact_f32, blocks(P.C.cs * NCOMP), kThr, s, u, P.C, cf);
    BSSN_LAUNCH(KC_CARTOON, k_axi_reconstruct_f32, grid, kAxiThreads, s, cf, u, P.C, A, w.uf, P.scs, sx, sy, 4, 4, 4,
                T);
    // the support is reconstructed in float alone: zero low words
    if (P.Gs.precision == kPrecisionF32Paired) {
        e = cudaMemsetAsync(w.uf + (long long)NCOMP * P.scs, 0, (size_t)NMIX * P.scs * sizeof(float), s);
        if (e != cudaSuccess) return e;
    }
    return launch_fill_periodic(w.uf, NCOMP, P.Gs, s);
}

cudaError_t compact_rhs(const CartoonPlan& P, const BssnParams* p, const double* u, double* kc, double* base,
                        cudaStream_t s, const AxiCol* T = nullptr) {
    double* us = base;
    double* ks = us + NCOMP * P.scs;
    const RhsWork w = carve_rhs_work(ks + NCOMP * P.scs, P.scs, P.with_mom);
    cudaError_t e;
    if (P.axi && float_form(P.Gs.precision)) {
        e = reconstruct_f32(P, p, u, us, w, s, T);
        if (e == cudaSuccess) e = launch_rhs_f32_prepared(us, ks, w, P.Gs, P.centre, s);
    } else {
        e = reconstruct(P, p, u, us, s, T);
        if (e == cudaSuccess) e = launch_rhs(us, ks, w, P.Gs, P.centre, s);
    }
    if (e == cudaSuccess) {
        const long long n = (long long)(P.C.nx - kCG) * P.C.nz * NCOMP;
        BSSN_LAUNCH(KC_CARTOON, k_collect, blocks(n), kThr, s, ks, P.scs, P.Gs.st[0], P.Gs.st[1], 4 + kCenter,
                    P.axi ? 4 : 4 + kCenter, kc, P.C);
        e = cudaGetLastError();
    }
    return e;
}

cudaError_t ghosts(const CartoonPlan& P, double* u, cudaStream_t s) {
    const long long n = (long long)kCG * P.C.nz * NCOMP;
    if (P.axi) BSSN_LAUNCH(KC_CARTOON, k_ghosts, blocks(n), kThr, s, u, P.C, -1.0, -1.0, 1.0);
    else BSSN_LAUNCH(KC_CARTOON, k_ghosts, blocks(n), kThr, s, u, P.C, -1.0, 1.0, 1.0);
    return cudaGetLastError();
}

// _prepare_stage: axisymmetric = projection, parity ghosts; spherical = symmetric
// subspace, projection, ghosts (positive samples; ghosts follow by parity)
cudaError_t prepare_compact(const CartoonPlan& P, double* u, cudaStream_t s) {
    cudaError_t e = cudaSuccess;
    if (!P.axi) {
        BSSN_LAUNCH(KC_CARTOON, k_sph_symmetry, blocks(P.C.nx), kThr, s, u, P.C.nx);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = launch_project(u, P.Gc, P.positive, s);
    if (e == cudaSuccess) e = ghosts(P, u, s);
    return e;
}

cudaError_t cartoon_step(const CartoonPlan& P, const BssnParams* p, double* u, double* base, cudaStream_t s) {
    double* comp = base + (long long)(2 * NCOMP + rhs_work_blocks(P.with_mom)) * P.scs;
    double* us = comp;
    double* kc = us + NCOMP * P.C.cs;
    double* acc = kc + NCOMP * P.C.cs;
    AxiCol* T = nullptr;
    if (P.axi) {
        // the geometry of every (x, plane pair) column, once for the four stages
        T = reinterpret_cast<AxiCol*>(acc + NCOMP * P.C.cs);
        const AxiGeom A{p->dx, p->xmin[2]};
        BSSN_LAUNCH(KC_CARTOON, k_axi_columns, blocks((long long)P.C.nx * kAxiPairs), kThr, s, P.C, A, T);
    }
    cudaError_t e = prepare_compact(P, u, s);
    for (int stage = 1; stage <= 4 && e == cudaSuccess; ++stage) {
        const double* src = stage == 1 ? u : us;
        e = compact_rhs(P, p, src, kc, base, s, T);
        double* out = stage == 4 ? u : us;
        if (e == cudaSuccess)
            e = launch_rk4_stage(u, kc, acc, out, P.Gc, P.positive, stage, p->dt, 0, /*project=*/0, s);
        if (e == cudaSuccess) e = prepare_compact(P, out, s);
    }
    return e;
}

}  // namespace
}  // namespace bssn

using namespace bssn;

extern "C" {

size_t bssn_cartoon_workspace_bytes(int32_t axisymmetric, const int32_t shape[3], const BssnParams* params) {
    CartoonPlan P;
    if (cartoon_plan(axisymmetric != 0, shape, params, P) != BSSN_OK) return 0;
    return cartoon_work_values(P) * sizeof(double);
}

int bssn_cartoon_fill_ghosts(int32_t axisymmetric, double* compact, const int32_t shape[3], void* stream) {
    if (!compact || !shape) return fail(BSSN_ERR_INVALID, "null pointer");
    CartoonPlan P;
    P.axi = axisymmetric != 0;
    P.C.nx = shape[0];
    P.C.nz = P.axi ? shape[2] : 1;
    P.C.cs = (long long)P.C.nx * P.C.nz;
    if (P.C.nx < 2 * kCG) return fail(BSSN_ERR_INVALID, "compact Cartoon state needs at least four positive samples");
    if (P.axi) return cuda_status(ghosts(P, compact, (cudaStream_t)stream), "bssn_cartoon_fill_ghosts");
    BSSN_LAUNCH(KC_CARTOON, k_sph_symmetry, blocks(P.C.nx), kThr, (cudaStream_t)stream, compact, P.C.nx);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = ghosts(P, compact, (cudaStream_t)stream);
    return cuda_status(e, "bssn_cartoon_fill_ghosts");
}

int bssn_cartoon_reconstruct(int32_t axisymmetric, const double* compact, double* support, const int32_t shape[3],
                             const BssnParams* params, void* stream) {
    if (!compact || !support) return fail(BSSN_ERR_INVALID, "null pointer");
    CartoonPlan P;
    int st = cartoon_plan(axisymmetric != 0, shape, params, P);
    if (st) return st;
    cudaStream_t s = (cudaStream_t)stream;
    if (P.axi) {
        const AxiGeom A{params->dx, params->xmin[2]};
        const long long dcs = (long long)P.C.nx * kSup * P.C.nz;
        const dim3 grid((unsigned)(P.C.nx * kAxiPairs), (unsigned)((P.C.nz + kAxiThreads - 1) / kAxiThreads));
        BSSN_LAUNCH(KC_CARTOON, k_axi_reconstruct, grid, kAxiThreads, s, compact, P.C, A, support, dcs,
                    (long long)kSup * P.C.nz, (long long)P.C.nz, 0, 0, 0, 0, nullptr);
    } else {
        const long long n = (long long)P.C.nx * kSup * kSup;
        BSSN_LAUNCH(KC_CARTOON, k_sph_reconstruct, blocks(n), kThr, s, compact, P.C.nx, params->dx, support, n,
                    (long long)kSup * kSup, (long long)kSup, 0, 0, 0);
    }
    return cuda_status(cudaGetLastError(), "bssn_cartoon_reconstruct");
}

int bssn_cartoon_rhs(int32_t axisymmetric, const double* compact, double* rhs, const int32_t shape[3],
                     const BssnParams* params, void* workspace, size_t workspace_bytes, void* stream) {
    if (!compact || !rhs) return fail(BSSN_ERR_INVALID, "null pointer");
    CartoonPlan P;
    int st = cartoon_plan(axisymmetric != 0, shape, params, P);
    if (st) return st;
    if (!workspace || workspace_bytes < cartoon_work_values(P) * sizeof(double))
        return fail(BSSN_ERR_WORKSPACE, "workspace missing or smaller than bssn_cartoon_workspace_bytes");
    cudaStream_t s = (cudaStream_t)stream;
    cudaError_t e = compact_rhs(P, params, compact, rhs, (double*)workspace, s);
    if (e == cudaSuccess) e = ghosts(P, rhs, s);
    return cuda_status(e, "bssn_cartoon_rhs");
}

int bssn_cartoon_rk4_step(int32_t axisymmetric, double* compact, const int32_t shape[3], const BssnParams* params,
                          int32_t steps, void* workspace, size_t workspace_bytes, void* stream) {
    if (!compact) return fail(BSSN_ERR_INVALID, "null pointer");
    if (steps < 0) return fail(BSSN_ERR_INVALID, "steps must be non-negative");
    CartoonPlan P;
    int st = cartoon_plan(axisymmetric != 0, shape, params, P);
    if (st) return st;
    if (!workspace || workspace_bytes < cartoon_work_values(P) * sizeof(double))
        return fail(BSSN_ERR_WORKSPACE, "workspace missing or smaller than bssn_cartoon_workspace_bytes");
    cudaError_t e = cudaSuccess;
    for (int n = 0; n < steps && e == cudaSuccess; ++n)
        e = cartoon_step(P, params, compact, (double*)workspace, (cudaStream_t)stream);
    return cuda_status(e, "bssn_cartoon_rk4_step");
}

int bssn_cartoon_constraints(int32_t axisymmetric, const double* compact, const int32_t shape[3],
                             const BssnParams* params, double* out, void* workspace, size_t workspace_bytes,
                             void* stream) {
    if (!compact || !out) return fail(BSSN_ERR_INVALID, "null pointer");
    CartoonPlan P;
    int st = cartoon_plan(axisymmetric != 0, shape, params, P);
    if (st) return st;
    if (!workspace || workspace_bytes < cartoon_constraint_values(P) * sizeof(double))
        return fail(BSSN_ERR_WORKSPACE, "workspace smaller than the Cartoon constraint need");
    cudaStream_t s = (cudaStream_t)stream;
    double* us = (double*)workspace;
    RhsWork w;
    w.d1 = us + NCOMP * P.scs;
    w.der = w.d1 + 3LL * NMIX * P.scs;
    double* fields = w.der + 24LL * P.scs;
    const long long n = P.centre.count;
    cudaError_t e = reconstruct(P, params, compact, us, s);
    if (e == cudaSuccess)
        e = launch_constraints(us, w, P.Gs, P.centre, fields, fields + n, fields + 4 * n, fields + 5 * n,
                               fields + 6 * n, s);
    if (e == cudaSuccess) {
        const long long m = 9LL * P.C.cs;
        BSSN_LAUNCH(KC_CARTOON, k_cons_compact, blocks(m), kThr, s, fields, P.C, out, P.axi ? 1 : 0);
        e = cudaGetLastError();
    }
    return cuda_status(e, "bssn_cartoon_constraints");
}

}  // extern "C"
