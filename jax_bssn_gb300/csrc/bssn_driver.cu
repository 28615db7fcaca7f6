// C ABI, geometry set-up and the point-wise kernels around the RHS:
// reference-layout import/export, periodic ghost fill, the algebraic
// projection (JAX_BSSN/evolution/time_evolve.py:94-141) and the RK4 stage
// epilogue (time_evolve.py:144-217).
//
// Stage combinations are evaluated with round-to-nearest intrinsics in the
// reference's order: u0 + (c*dt)*k for the stages, the accumulator
// ((k1 + 2 k2) + 2 k3) + k4 and u0 + (dt/6)*sum (serial, tiled and Cartoon
// steppers) or u0 + (dt*sum)/6 (JAX_BSSN/fmr/tiled.py:195-196).  Together
// with the bit-exact projection this keeps the evolved state identical to the
// float64 reference wherever the RHS agrees to the last bit.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>

#include "../../include/bssn_gb300.h"
#include "bssn_driver.h"
#include "bssn_fields.cuh"
#include "bssn_kernels.h"
#include "bssn_profile.h"

namespace bssn {

static thread_local std::string g_last_error;

int fail(int code, const std::string& msg) {
    g_last_error = msg;
    return code;
}

int cuda_status(cudaError_t e, const char* where) {
    if (e == cudaSuccess) return BSSN_OK;
    return fail(BSSN_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
}

constexpr int kThreads = 256;
static inline unsigned nblocks(long long n) { return (unsigned)((n + kThreads - 1) / kThreads); }

// ---------------------------------------------------------------------------
// geometry
// ---------------------------------------------------------------------------
int validate_params(const BssnParams* p) {
    if (p == nullptr) return fail(BSSN_ERR_INVALID, "params is null");
    if (!(std::isfinite(p->dx) && p->dx > 0.0)) return fail(BSSN_ERR_INVALID, "dx must be finite and positive");
    if (!std::isfinite(p->dt)) return fail(BSSN_ERR_INVALID, "dt must be finite");
    for (int f = 0; f < 6; ++f)
        if (p->bc[f] != 0 && p->bc[f] != 1)
            return fail(BSSN_ERR_INVALID, "boundary codes must be 0 (periodic) or 1 (Sommerfeld)");
    if (p->gauge != 0 && p->gauge != 1) return fail(BSSN_ERR_INVALID, "gauge must be 0 or 1");
    if (p->precision != BSSN_PRECISION_F64 && p->precision != BSSN_PRECISION_F32 &&
        p->precision != BSSN_PRECISION_F32_PAIRED)
        return fail(BSSN_ERR_INVALID,
                    "precision must be BSSN_PRECISION_F64, BSSN_PRECISION_F32 or BSSN_PRECISION_F32_PAIRED");
    return BSSN_OK;
}

// Geometry of an array of extent S embedded at padded offset `org` in a
// padded block of extent P.  The owned range follows the reference's
// guard_cells/owned_shape (JAX_BSSN/evolution/spatial_derivatives.py:18-41),
// the Sommerfeld mask follows boundaries.py:44-71.
int make_geo(const BssnParams* p, const int S[3], const int org[3], const int P[3], Geo& G) {
    std::memset(&G, 0, sizeof(G));
    const bool owned_given = p->owned_shape[0] >= 0;
    for (int d = 0; d < 3; ++d) {
        Axis& a = G.ax[d];
        a.P = P[d];
        a.org = org[d];
        a.lo = org[d];
        a.hi = org[d] + S[d];
        const int count = owned_given ? p->owned_shape[d] : S[d];
        a.start = org[d] + p->guard_cells;
        a.end = a.start + count;
        if (count < 1 || p->guard_cells < 0 || p->guard_cells + count > S[d])
            return fail(BSSN_ERR_INVALID, "owned range does not fit the array");
        const int lcode = p->bc[2 * d], rcode = p->bc[2 * d + 1];
        const bool lown = p->owned_faces[2 * d] != 0, rown = p->owned_faces[2 * d + 1] != 0;
        a.lbc = (lcode == kSommerfeld) && lown;
        a.rbc = (rcode == kSommerfeld) && rown;
        const bool physical_global = lcode == kSommerfeld || rcode == kSommerfeld;
        a.q = physical_global ? 1.0 : p->mad_q;
        a.omq = 1.0 - a.q;
        a.mad = a.q != 1.0;
        if (p->reduced_axes[d] >= 0) a.reduced = p->reduced_axes[d] != 0;
        else a.reduced = owned_given ? (count == 1) : 0;
        const bool counts_ok = owned_given ? count > 1 : true;
        a.slo = a.lbc && counts_ok;
        a.shi = a.rbc && counts_ok;
        a.xmin = p->xmin[d];
        a.fq = static_cast<float>(a.q);
        a.fomq = static_cast<float>(a.omq);
        if ((a.lbc || a.rbc) && !a.reduced && count < 8)
            return fail(BSSN_ERR_INVALID, "Sommerfeld/KO closures require eight owned samples along the axis");
        if (a.lo < 4 || a.hi > P[d] - 4)
            return fail(BSSN_ERR_INVALID, "padded block needs four samples of margin around the compute range");
    }
    G.st[2] = 1;
    G.st[1] = P[2];
    G.st[0] = (long long)P[1] * P[2];
    G.cs = (long long)P[0] * P[1] * P[2];
    G.ninst = 1;
    G.istride = G.cs;
    const double dx = p->dx;
    G.dx = dx;
    G.inv_dx = 1.0 / dx;
    G.inv_12dx = 1.0 / (12.0 * dx);
    G.inv_60dx = 1.0 / (60.0 * dx);
    G.inv_12dx2 = 1.0 / (12.0 * (dx * dx));
    G.inv_dx2 = 1.0 / (dx * dx);
    G.inv_dx6h5 = std::pow(dx, 5.0) / std::pow(dx, 6.0);
    G.nu64 = p->nu / 64.0;
    G.d1a = (2.0 / 3.0) * G.inv_dx;
    G.d1b = (-1.0 / 12.0) * G.inv_dx;
    G.ko_scale = G.nu64 * G.inv_dx6h5;
    G.eta = p->eta;
    G.kappa = p->kappa;
    G.g = p->g;
    G.dt = p->dt;
    G.gauge = p->gauge;
    G.zero_shift = p->zero_shift;
    G.any_sommerfeld = 0;
    for (int f = 0; f < 6; ++f) G.any_sommerfeld |= (p->bc[f] == kSommerfeld);
    G.precision = p->precision;
    G.gf.inv_dx = static_cast<float>(G.inv_dx);
    G.gf.inv_12dx = static_cast<float>(G.inv_12dx);
    G.gf.inv_60dx = static_cast<float>(G.inv_60dx);
    G.gf.inv_12dx2 = static_cast<float>(G.inv_12dx2);
    G.gf.inv_dx2 = static_cast<float>(G.inv_dx2);
    G.gf.inv_dx6h5 = static_cast<float>(G.inv_dx6h5);
    G.gf.nu64 = static_cast<float>(G.nu64);
    G.gf.d1a = static_cast<float>(G.d1a);
    G.gf.d1b = static_cast<float>(G.d1b);
    G.gf.ko_scale = static_cast<float>(G.ko_scale);
    G.gf.eta = static_cast<float>(G.eta);
    G.gf.kappa = static_cast<float>(G.kappa);
    G.gf.g = static_cast<float>(G.g);
    return BSSN_OK;
}

Box box_of(const Geo& G) {
    Box b;
    b.count = 1;
    for (int d = 0; d < 3; ++d) {
        b.lo[d] = G.ax[d].lo;
        b.n[d] = G.ax[d].hi - G.ax[d].lo;
        b.count *= b.n[d];
    }
    return b;
}

Box full_box(const Geo& G) {
    Box b;
    b.count = 1;
    for (int d = 0; d < 3; ++d) {
        b.lo[d] = 0;
        b.n[d] = G.ax[d].P;
        b.count *= b.n[d];
    }
    return b;
}

RhsWork carve_rhs_work(double* base, long long cs, bool with_mom) {
    RhsWork w;
    w.d1 = base;
    if (with_mom) {
        w.der = base + (long long)(3 * (NMIX + NMIX_MOM)) * cs;
        w.damp = w.der + 24LL * cs;
    }
    // FP32 views of the same memory: 21 perturbations, the low words of the
    // NMIX second-derivative fields, then 3 * nfield (+ 24 + 6) floats per
    // sample -- within the 3 * nfield (+ 24 + 6) doubles of the FP64 layout.
    const int nfield = with_mom ? NMIX + NMIX_MOM : NMIX;
    static_assert(NCOMP + NMIX + 3 * NMIX <= 2 * 3 * NMIX, "FP32 views must fit the FP64 scratch");
    static_assert(NCOMP + NMIX + 3 * (NMIX + NMIX_MOM) + 30 <= 2 * (3 * (NMIX + NMIX_MOM) + 30),
                  "FP32 views must fit the FP64 scratch");
    w.uf = reinterpret_cast<float*>(base);
    w.d1f = w.uf + (long long)(NCOMP + NMIX) * cs;
    if (with_mom) {
        w.derf = w.d1f + (long long)(3 * nfield) * cs;
        w.dampf = w.derf + 24LL * cs;
    }
    return w;
}

// ---------------------------------------------------------------------------
// point-wise kernels
// ---------------------------------------------------------------------------
struct Leaves {
    const double* f[7];
};
struct LeavesOut {
    double* f[7];
};

__device__ __forceinline__ void leaf_of(int comp, int& leaf, int& idx) {
    // component -> (leaf, flat component index inside the leaf) in the reference layout
    if (comp < 6) { leaf = 0; const int i = comp < 3 ? 0 : (comp < 5 ? 1 : 2); const int j = comp < 3 ? comp : (comp < 5 ? comp - 2 : 2); idx = 3 * i + j; }
    else if (comp == CW) { leaf = 1; idx = 0; }
    else if (comp < CK) { leaf = 2; const int c = comp - AXX; const int i = c < 3 ? 0 : (c < 5 ? 1 : 2); const int j = c < 3 ? c : (c < 5 ? c - 2 : 2); idx = 3 * i + j; }
    else if (comp == CK) { leaf = 3; idx = 0; }
    else if (comp < CALPHA) { leaf = 4; idx = comp - GTX; }
    else if (comp == CALPHA) { leaf = 5; idx = 0; }
    else { leaf = 6; idx = comp - BX; }
}

// Reference-layout conversions run one thread per sample of a z row: grid
// (z blocks, rows, components), blocks striding over the rows, so a thread
// finds its sample with one 32-bit division per row.  r is the sample's index
// in the reference layout (x, y, z order of the region).
constexpr int kRowThreads = 128;
dim3 row_grid(const Box& B, int ncomp) {
    const long long rows = (long long)B.n[0] * B.n[1];
    return dim3((unsigned)((B.n[2] + kRowThreads - 1) / kRowThreads), (unsigned)std::max(1LL, std::min(rows, 65535LL)),
                (unsigned)ncomp);
}
template <typename F>
__device__ __forceinline__ void for_rows(const Box& B, F f) {
    const int z = blockIdx.x * blockDim.x + threadIdx.x;
    if (z >= B.n[2]) return;
    const int rows = B.n[0] * B.n[1];
    for (int row = blockIdx.y; row < rows; row += gridDim.y) {
        const int x = row / B.n[1], y = row - x * B.n[1];
        const int ix[3] = {B.lo[0] + x, B.lo[1] + y, B.lo[2] + z};
        f(ix, (long long)row * B.n[2] + z);
    }
}

// reference layout (shape S) -> padded block at org
__global__ void k_import(Leaves in, double* __restrict__ u, Geo G, Box region, long long npts) {
    const int comp = blockIdx.z;
    int leaf, idx;
    leaf_of(comp, leaf, idx);
    const double* src = in.f[leaf] + idx * npts;
    double* dst = u + comp * G.cs;
    for_rows(region, [&](const int (&ix)[3], long long r) { dst[lin(G, ix)] = src[r]; });
}

// padded block -> reference layout; symmetric tensors written to both halves
__global__ void k_export(const double* __restrict__ u, LeavesOut out, Geo G, Box region, long long npts) {
    const int comp = blockIdx.z;
    int leaf, idx;
    leaf_of(comp, leaf, idx);
    const double* src = u + comp * G.cs;
    double* dst = out.f[leaf] + idx * npts;
    const int i = idx / 3, j = idx % 3;
    double* mirror = ((leaf == 0 || leaf == 2) && i != j) ? out.f[leaf] + (3 * j + i) * npts : nullptr;
    for_rows(region, [&](const int (&ix)[3], long long r) {
        const double v = src[lin(G, ix)];
        dst[r] = v;
        if (mirror) mirror[r] = v;
    });
}

// Matter sources in the reference layout -> a padded block of kMatterComps
// components: rho, S_x, S_y, S_z, then the upper triangle of S_ij.
__global__ void k_import_matter(const double* __restrict__ rho, const double* __restrict__ Si,
                                const double* __restrict__ Sij, double* __restrict__ m, Geo G, Box region,
                                long long npts) {
    const int comp = blockIdx.z;
    const double* src;
    if (comp == 0) {
        src = rho;
    } else if (comp < 4) {
        src = Si + (comp - 1) * npts;
    } else {
        constexpr int ij[6][2] = {{0, 0}, {0, 1}, {0, 2}, {1, 1}, {1, 2}, {2, 2}};
        const int s = comp - 4;
        src = Sij + (3 * ij[s][0] + ij[s][1]) * npts;
    }
    double* dst = m + comp * G.cs;
    for_rows(region, [&](const int (&ix)[3], long long r) { dst[lin(G, ix)] = src[r]; });
}

// Periodic wrap of the array region [lo, lo+n) into every other padded sample
// (np.roll semantics of the reference on an unpadded array, and the self-wrap
// of a single tile, JAX_BSSN/parallel/communication.py:45-52).  Samples beyond
// an axis whose two faces are both Sommerfeld-closed (bit d of `closed`) are
// left alone: on such an axis the one-sided closures cover the three outer
// rows and every interior stencil stays inside the region, so nothing reads
// them.
template <typename T>
__global__ void k_fill_periodic(T* __restrict__ u, int ncomp, Geo G, Box region, Box all, int closed) {
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= box_threads(G, all)) return;
    const long long off = instance_offset(G, all, t);
    int ix[3];
    all.coords(t, ix);
    bool inside = true;
    int src[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        int rel = ix[d] - region.lo[d];
        const bool out = rel < 0 || rel >= region.n[d];
        if (out && ((closed >> d) & 1)) return;
        if (out) inside = false;
        rel %= region.n[d];
        if (rel < 0) rel += region.n[d];
        src[d] = region.lo[d] + rel;
    }
    if (inside) return;
    const long long dst = lin(G, ix) + off, s = lin(G, src) + off;
    for (int c = 0; c < ncomp; ++c) u[c * G.cs + dst] = u[c * G.cs + s];
}

// Bit-exact algebraic projection of one point held in registers
// (JAX_BSSN/evolution/time_evolve.py:94-141).  At's trace uses the
// reference's Cholesky inverse in its rounding order, not a cheaper cofactor
// form: a one-ulp change of At flips, here and there, the rounding of gt's
// next RK4 combination, and the Ricci tensor's 1/dx^2 gain turns that ulp of
// gt into ~1e-12 of At within three steps (measured at 32^3).
__device__ __forceinline__ void project_point(double (&g)[6], double (&A)[6]) {
    const double s = inv_cbrt_cr(det_sym_rn(g));
#pragma unroll
    for (int c = 0; c < 6; ++c) g[c] = __dmul_rn(g[c], s);
    double gi[6];
    inverse_metric_rn(g, gi);
    // trace gt^ij At_ij over all nine (i, j) in row-major order
    double tr = __dmul_rn(gi[0], A[0]);
    tr = __dadd_rn(tr, __dmul_rn(gi[1], A[1]));
    tr = __dadd_rn(tr, __dmul_rn(gi[2], A[2]));
    tr = __dadd_rn(tr, __dmul_rn(gi[1], A[1]));
    tr = __dadd_rn(tr, __dmul_rn(gi[3], A[3]));
    tr = __dadd_rn(tr, __dmul_rn(gi[4], A[4]));
    tr = __dadd_rn(tr, __dmul_rn(gi[2], A[2]));
    tr = __dadd_rn(tr, __dmul_rn(gi[4], A[4]));
    tr = __dadd_rn(tr, __dmul_rn(gi[5], A[5]));
#pragma unroll
    for (int c = 0; c < 6; ++c) A[c] = __dadd_rn(A[c], -__dmul_rn(__dmul_rn(1.0 / 3.0, g[c]), tr));
}

// Projection of the FP32-arithmetic form.  The state stays FP64; the
// correction is formed cheaply: det(gt) with FMAs, det^(-1/3) by its binomial
// series (|det - 1| < 1e-3, truncation below 2e-16) or rcbrt, and the trace
// gt^ij At_ij in float (the trace is itself a small correction, so float's
// relative precision is kept relative to it).
__device__ __forceinline__ void project_point_light(double (&g)[6], double (&A)[6]) {
    const double det = g[0] * (g[3] * g[5] - g[4] * g[4]) - g[1] * (g[1] * g[5] - g[4] * g[2])
                       + g[2] * (g[1] * g[4] - g[3] * g[2]);
    const double e = det - 1.0;
    const double s = fabs(e) < 1.0e-3
                         ? 1.0 + e * (-1.0 / 3.0 + e * (2.0 / 9.0 + e * (-14.0 / 81.0 + e * (35.0 / 243.0))))
                         : rcbrt(det);
    float gf[6], gi[6];
#pragma unroll
    for (int c = 0; c < 6; ++c) {
        g[c] *= s;
        gf[c] = static_cast<float>(g[c]);
    }
    inverse_metric(gf, gi);
    float Af[6];
#pragma unroll
    for (int c = 0; c < 6; ++c) Af[c] = static_cast<float>(A[c]);
    const float tr = gi[0] * Af[0] + gi[3] * Af[3] + gi[5] * Af[5]
                     + 2.0f * (gi[1] * Af[1] + gi[2] * Af[2] + gi[4] * Af[4]);
#pragma unroll
    for (int c = 0; c < 6; ++c) A[c] -= static_cast<double>((1.0f / 3.0f) * gf[c] * tr);
}

__device__ __forceinline__ void project_form(double (&g)[6], double (&A)[6], int precision) {
    if (float_form(precision)) project_point_light(g, A);
    else project_point(g, A);
}

__global__ void k_project(double* __restrict__ u, Geo G, Box B) {
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= box_threads(G, B)) return;
    const long long off = instance_offset(G, B, t);
    int ix[3];
    B.coords(t, ix);
    const long long p = lin(G, ix) + off, cs = G.cs;
    double g[6], A[6];
#pragma unroll
    for (int c = 0; c < 6; ++c) { g[c] = u[(GXX + c) * cs + p]; A[c] = u[(AXX + c) * cs + p]; }
    project_form(g, A, G.precision);
#pragma unroll
    for (int c = 0; c < 6; ++c) { u[(GXX + c) * cs + p] = g[c]; u[(AXX + c) * cs + p] = A[c]; }
}

// Projection in place on the reference layout (all samples).
__global__ void k_project_ref(LeavesOut f, long long npts) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= npts) return;
    constexpr int ij[6][2] = {{0, 0}, {0, 1}, {0, 2}, {1, 1}, {1, 2}, {2, 2}};
    double g[6], A[6];
#pragma unroll
    for (int c = 0; c < 6; ++c) {
        g[c] = f.f[0][(3 * ij[c][0] + ij[c][1]) * npts + t];
        A[c] = f.f[2][(3 * ij[c][0] + ij[c][1]) * npts + t];
    }
    project_point(g, A);
#pragma unroll
    for (int c = 0; c < 6; ++c) {
        const int a = ij[c][0], b = ij[c][1];
        f.f[0][(3 * a + b) * npts + t] = g[c];
        f.f[0][(3 * b + a) * npts + t] = g[c];
        f.f[2][(3 * a + b) * npts + t] = A[c];
        f.f[2][(3 * b + a) * npts + t] = A[c];
    }
}

// RK4 stage epilogue.  stage 1..3: out = u0 + h*k, acc updated; stage 4:
// out = u0 + (dt/6)*(acc + k)  [final_form 0]  or  (dt*(acc + k))/6  [1].
// Light = false: every operation rounded as the reference orders it and the
// bit-exact projection.  Light = true (FP32-arithmetic form): the same
// combination with FMAs, a multiply by 1/6 and the light projection.
template <bool Light>
__global__ void k_rk4_stage(const double* __restrict__ u0, const double* __restrict__ k,
                            double* __restrict__ acc, double* __restrict__ out, Geo G, Box B,
                            int stage, double h, double dt, int final_form, int project) {
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= box_threads(G, B)) return;
    const long long off = instance_offset(G, B, t);
    int ix[3];
    B.coords(t, ix);
    const long long p = lin(G, ix) + off, cs = G.cs;
    double v[NCOMP];
#pragma unroll
    for (int c = 0; c < NCOMP; ++c) {
        const long long q = c * cs + p;
        const double kv = k[q];
        if constexpr (Light) {
            if (stage < 4) {
                v[c] = fma(h, kv, u0[q]);
                acc[q] = (stage == 1) ? kv : fma(2.0, kv, acc[q]);
            } else {
                v[c] = fma(dt * (1.0 / 6.0), acc[q] + kv, u0[q]);
            }
        } else {
            if (stage < 4) {
                v[c] = __dadd_rn(u0[q], __dmul_rn(h, kv));
                acc[q] = (stage == 1) ? kv : __fma_rn(2.0, kv, acc[q]);  // 2k is exact: same bits as mul + add
            } else {
                const double s = __dadd_rn(acc[q], kv);
                const double inc = final_form ? div6_rn(__dmul_rn(dt, s)) : __dmul_rn(dt / 6.0, s);
                v[c] = __dadd_rn(u0[q], inc);
            }
        }
    }
    if (project) {
        double g[6], A[6];
#pragma unroll
        for (int c = 0; c < 6; ++c) { g[c] = v[GXX + c]; A[c] = v[AXX + c]; }
        if constexpr (Light) project_point_light(g, A);
        else project_point(g, A);
#pragma unroll
        for (int c = 0; c < 6; ++c) { v[GXX + c] = g[c]; v[AXX + c] = A[c]; }
    }
#pragma unroll
    for (int c = 0; c < NCOMP; ++c) out[c * cs + p] = v[c];
}

__global__ void k_count_nonfinite(const double* __restrict__ u, Geo G, Box B, int* flag) {
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= box_threads(G, B)) return;
    const long long off = instance_offset(G, B, t);
    int ix[3];
    B.coords(t, ix);
    const long long p = lin(G, ix) + off;
    int bad = 0;
    for (int c = 0; c < NCOMP; ++c) bad += !isfinite(u[c * G.cs + p]);
    if (bad) atomicAdd(flag, bad);
}

__global__ void k_zero(double* __restrict__ u, long long n) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) u[t] = 0.0;
}

// ---------------------------------------------------------------------------
// launchers shared by the C ABI, FMR and Cartoon drivers
// ---------------------------------------------------------------------------
template <typename T>
static cudaError_t fill_periodic(T* u, int ncomp, const Geo& G, cudaStream_t s) {
    const Box region = box_of(G);
    const Box all = full_box(G);
    int closed = 0;
    for (int d = 0; d < 3; ++d) {
        const Axis& a = G.ax[d];
        // both faces closed and owned by this region: no stencil leaves it
        if (!a.reduced && a.lbc && a.rbc && a.lo == a.start && a.hi == a.end) closed |= 1 << d;
    }
    if (closed == 7) return cudaSuccess;
    BSSN_LAUNCH(KC_FILL, k_fill_periodic<T>, nblocks(box_threads(G, all)), kThreads, s, u, ncomp, G, region, all,
                closed);
    return cudaGetLastError();
}

cudaError_t launch_fill_periodic(double* u, int ncomp, const Geo& G, cudaStream_t s) {
    return fill_periodic(u, ncomp, G, s);
}

cudaError_t launch_fill_periodic(float* u, int ncomp, const Geo& G, cudaStream_t s) {
    return fill_periodic(u, ncomp, G, s);
}

cudaError_t launch_project(double* u, const Geo& G, const Box& B, cudaStream_t s) {
    BSSN_LAUNCH(KC_PROJECT, k_project, nblocks(box_threads(G, B)), kThreads, s, u, G, B);
    return cudaGetLastError();
}

cudaError_t launch_rk4_stage(const double* u0, const double* k, double* acc, double* out, const Geo& G,
                             const Box& B, int stage, double dt, int final_form, int project,
                             cudaStream_t s) {
    const double h = stage == 3 ? dt : 0.5 * dt;
    if (float_form(G.precision))
        BSSN_LAUNCH(KC_STAGE, k_rk4_stage<true>, nblocks(box_threads(G, B)), kThreads, s, u0, k, acc, out, G, B, stage, h, dt,
                    final_form, project);
    else
        BSSN_LAUNCH(KC_STAGE, k_rk4_stage<false>, nblocks(box_threads(G, B)), kThreads, s, u0, k, acc, out, G, B, stage, h, dt,
                    final_form, project);
    return cudaGetLastError();
}

cudaError_t launch_zero(double* u, long long n, cudaStream_t s) {
    BSSN_LAUNCH(KC_OTHER, k_zero, nblocks(n), kThreads, s, u, n);
    return cudaGetLastError();
}

// One classical RK4 step of the state u0 (in place), with the RHS over the
// box B and the projection both before the first stage (serial stepper) and
// after every combination.
cudaError_t rk4_step_patch(double* u0, double* ustage, double* k, double* acc, const RhsWork& w,
                           const Geo& G, const Box& B, bool fill, int final_form, cudaStream_t s,
                           const LowerTriangle* lower) {
    cudaError_t e;
    for (int stage = 1; stage <= 4; ++stage) {
        const double* src = stage == 1 ? u0 : ustage;
        if (fill && (e = launch_fill_periodic(const_cast<double*>(src), NCOMP, G, s)) != cudaSuccess) return e;
        if ((e = launch_rhs(src, k, w, G, B, s)) != cudaSuccess) return e;
        if (lower) {
            if ((e = launch_lower_triangle(src, w, *lower, G, B, stage, s)) != cudaSuccess) return e;
            // periodic axes: the next reader's ghosts
            if ((e = launch_fill_periodic(lower_triangle_output(*lower, stage), 6, G, s)) != cudaSuccess) return e;
        }
        double* out = stage == 4 ? u0 : ustage;
        if ((e = launch_rk4_stage(u0, k, acc, out, G, B, stage, G.dt, final_form, 1, s)) != cudaSuccess) return e;
    }
    return cudaSuccess;
}

// delta_ij = T_ji - T_ij (i < j) of a reference-layout input's At and gt,
// on the closure-row shell (zero elsewhere: an input whose triangles differ
// in the interior evolves with its upper triangle there), and the lower
// triangles of an output as their upper triangles plus delta.
__device__ __forceinline__ bool in_closure_shell(const Geo& G, const int (&ix)[3]) {
    bool shell = false;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        const Axis& a = G.ax[d];
        if (a.reduced) continue;
        shell = shell || (a.lbc && ix[d] < a.start + kClosureRows) || (a.rbc && ix[d] >= a.end - kClosureRows);
    }
    return shell;
}

__global__ void k_import_lower(const double* __restrict__ A, const double* __restrict__ g, double* __restrict__ delta,
                               float* __restrict__ copy, float* __restrict__ other, Geo G, Box region,
                               long long npts) {
    const int k = blockIdx.z;
    constexpr int pairs[3][2] = {{0, 1}, {0, 2}, {1, 2}};
    const int i = pairs[k % 3][0], j = pairs[k % 3][1];
    const double* T = k < 3 ? A : g;
    for_rows(region, [&](const int (&ix)[3], long long r) {
        const double d = in_closure_shell(G, ix) ? T[(3 * j + i) * npts + r] - T[(3 * i + j) * npts + r] : 0.0;
        const long long q = k * G.cs + lin(G, ix);
        delta[q] = d;
        copy[q] = (float)d;    // stage 1 reads it
        other[q] = 0.0f;       // off the shell, stage values stay zero
    });
}

__global__ void k_export_lower(double* __restrict__ A, double* __restrict__ g, const double* __restrict__ delta,
                               Geo G, Box region, long long npts) {
    const int k = blockIdx.z;
    constexpr int pairs[3][2] = {{0, 1}, {0, 2}, {1, 2}};
    const int i = pairs[k % 3][0], j = pairs[k % 3][1];
    double* T = k < 3 ? A : g;
    for_rows(region, [&](const int (&ix)[3], long long r) {
        T[(3 * j + i) * npts + r] = T[(3 * i + j) * npts + r] + delta[k * G.cs + lin(G, ix)];
    });
}

}  // namespace bssn

// ===========================================================================
// C ABI
// ===========================================================================
using namespace bssn;

namespace {

constexpr int kMargin = 4;

struct RefLayout {
    int S[3];
    int org[3];
    int P[3];
    long long npts;
    long long cs;
};

int ref_layout(const int32_t shape[3], RefLayout& L) {
    if (shape == nullptr) return fail(BSSN_ERR_INVALID, "shape is null");
    L.npts = 1;
    L.cs = 1;
    for (int d = 0; d < 3; ++d) {
        if (shape[d] < 1) return fail(BSSN_ERR_INVALID, "array extents must be positive");
        L.S[d] = shape[d];
        L.org[d] = kMargin;
        L.P[d] = shape[d] + 2 * kMargin;
        L.npts *= shape[d];
        L.cs *= L.P[d];
    }
    return BSSN_OK;
}

bool fields_ok(const BssnFields* f) {
    return f && f->conformal_metric && f->conformal_factor && f->traceless_K && f->trace_K &&
           f->conformal_connection && f->lapse && f->shift;
}

Leaves leaves_in(const BssnFields* f) {
    return Leaves{{f->conformal_metric, f->conformal_factor, f->traceless_K, f->trace_K,
                   f->conformal_connection, f->lapse, f->shift}};
}
LeavesOut leaves_out(BssnFields* f) {
    return LeavesOut{{f->conformal_metric, f->conformal_factor, f->traceless_K, f->trace_K,
                      f->conformal_connection, f->lapse, f->shift}};
}

// The reference-layout RK4 call carries the reference's At and gt lower
// triangles (launch_lower_triangle) in the plain FP64 form when a face is
// Sommerfeld.
bool carries_lower_triangle(const BssnParams* p) {
    if (!p || p->precision != BSSN_PRECISION_F64) return false;
    for (int f = 0; f < 6; ++f)
        if (p->bc[f] == 1) return true;
    return false;
}

size_t ref_workspace_values(int op, const RefLayout& L, bool with_mom, bool lower = false) {
    if (op == BSSN_OP_CONSTRAINTS) return (size_t)(NCOMP + 3 * NMIX + 24) * (size_t)L.cs;
    size_t blocks = (op == BSSN_OP_RK4 ? 4 * NCOMP : 2 * NCOMP) + rhs_work_blocks(with_mom);
    if (op == BSSN_OP_RHS_MATTER) blocks += kMatterComps;
    if (op == BSSN_OP_RK4 && lower) blocks += kLowerTriangleBlocks;
    return blocks * (size_t)L.cs;
}

bool matter_given(const BssnMatter* m) {
    return m && (m->energy_density || m->momentum_density || m->spatial_stress);
}

}  // namespace

extern "C" {

const char* bssn_last_error(void) { return g_last_error.c_str(); }

int bssn_abi_version(void) { return BSSN_ABI_VERSION; }

size_t bssn_workspace_bytes(int op, const int32_t shape[3], const BssnParams* params) {
    RefLayout L;
    if (ref_layout(shape, L) != BSSN_OK) return 0;
    const bool with_mom = params && params->kappa != 0.0;
    return ref_workspace_values(op, L, with_mom, carries_lower_triangle(params)) * sizeof(double);
}

int bssn_rhs(const BssnFields* in, BssnFields* out, const int32_t shape[3], const BssnParams* params,
             const BssnMatter* matter, void* workspace, size_t workspace_bytes, void* stream) {
    if (!fields_ok(in) || !fields_ok(out)) return fail(BSSN_ERR_INVALID, "null field pointer");
    const bool with_matter = matter_given(matter);
    if (with_matter && !(matter->energy_density && matter->momentum_density && matter->spatial_stress))
        return fail(BSSN_ERR_INVALID, "matter sources need energy_density, momentum_density and spatial_stress");
    int st = validate_params(params);
    if (st) return st;
    RefLayout L;
    if ((st = ref_layout(shape, L))) return st;
    Geo G;
    if ((st = make_geo(params, L.S, L.org, L.P, G))) return st;
    const bool with_mom = params->kappa != 0.0;
    const int op = with_matter ? BSSN_OP_RHS_MATTER : BSSN_OP_RHS;
    if (!workspace || workspace_bytes < ref_workspace_values(op, L, with_mom) * sizeof(double))
        return fail(BSSN_ERR_WORKSPACE, with_matter
                    ? "workspace missing or smaller than bssn_workspace_bytes(BSSN_OP_RHS_MATTER)"
                    : "workspace missing or smaller than bssn_workspace_bytes(BSSN_OP_RHS)");
    cudaStream_t s = (cudaStream_t)stream;
    double* u = (double*)workspace;
    double* k = u + NCOMP * L.cs;
    RhsWork w = carve_rhs_work(k + NCOMP * L.cs, L.cs, with_mom);
    const Box region = box_of(G);
    BSSN_LAUNCH(KC_IMPORT, k_import, row_grid(region, NCOMP), kRowThreads, s, leaves_in(in), u, G, region, L.npts);
    cudaError_t e = launch_fill_periodic(u, NCOMP, G, s);
    if (e == cudaSuccess && with_matter) {
        double* m = k + (long long)(NCOMP + rhs_work_blocks(with_mom)) * L.cs;
        BSSN_LAUNCH(KC_IMPORT, k_import_matter, row_grid(region, kMatterComps), kRowThreads, s,
                    matter->energy_density, matter->momentum_density, matter->spatial_stress, m, G, region, L.npts);
        e = launch_fill_periodic(m, kMatterComps, G, s);
        w.mat = m;
    }
    if (e == cudaSuccess) e = launch_rhs(u, k, w, G, region, s);
    if (e == cudaSuccess) {
        BSSN_LAUNCH(KC_EXPORT, k_export, row_grid(region, NCOMP), kRowThreads, s, k, leaves_out(out), G, region, L.npts);
        e = cudaGetLastError();
    }
    return cuda_status(e, "bssn_rhs");
}

int bssn_project(BssnFields* state, const int32_t shape[3], void* stream) {
    if (!fields_ok(state)) return fail(BSSN_ERR_INVALID, "null field pointer");
    RefLayout L;
    int st = ref_layout(shape, L);
    if (st) return st;
    BSSN_LAUNCH(KC_PROJECT, k_project_ref, nblocks(L.npts), kThreads, (cudaStream_t)stream, leaves_out(state), L.npts);
    return cuda_status(cudaGetLastError(), "bssn_project");
}

int bssn_rk4_step(BssnFields* state, const int32_t shape[3], const BssnParams* params, int32_t steps,
                  void* workspace, size_t workspace_bytes, void* stream) {
    if (!fields_ok(state)) return fail(BSSN_ERR_INVALID, "null field pointer");
    if (steps < 0) return fail(BSSN_ERR_INVALID, "steps must be non-negative");
    int st = validate_params(params);
    if (st) return st;
    RefLayout L;
    if ((st = ref_layout(shape, L))) return st;
    Geo G;
    if ((st = make_geo(params, L.S, L.org, L.P, G))) return st;
    const bool with_mom = params->kappa != 0.0;
    const bool lower = carries_lower_triangle(params);
    if (!workspace || workspace_bytes < ref_workspace_values(BSSN_OP_RK4, L, with_mom, lower) * sizeof(double))
        return fail(BSSN_ERR_WORKSPACE, "workspace missing or smaller than bssn_workspace_bytes(BSSN_OP_RK4)");
    cudaStream_t s = (cudaStream_t)stream;
    double* u0 = (double*)workspace;
    double* us = u0 + NCOMP * L.cs;
    double* k = us + NCOMP * L.cs;
    double* acc = k + NCOMP * L.cs;
    RhsWork w = carve_rhs_work(acc + NCOMP * L.cs, L.cs, with_mom);
    LowerTriangle lt;
    lt.delta = acc + (NCOMP + rhs_work_blocks(with_mom)) * L.cs;
    lt.acc = (float*)(lt.delta + 6 * L.cs);
    lt.stage[0] = lt.acc + 6 * L.cs;
    lt.stage[1] = lt.stage[0] + 6 * L.cs;
    const Box region = box_of(G);
    BSSN_LAUNCH(KC_IMPORT, k_import, row_grid(region, NCOMP), kRowThreads, s, leaves_in(state), u0, G, region, L.npts);
    cudaError_t e = cudaGetLastError();
    if (lower && e == cudaSuccess) {
        // delta, its FP32 copy (stage 1's input) and zero stage values over
        // the owned box; stencils reach no padding along closed axes
        BSSN_LAUNCH(KC_IMPORT, k_import_lower, row_grid(region, 6), kRowThreads, s, state->traceless_K,
                    state->conformal_metric, lt.delta, lower_triangle_input(lt, 1), lower_triangle_output(lt, 1), G,
                    region, L.npts);
        e = cudaGetLastError();
        if (e == cudaSuccess) e = launch_fill_periodic(lower_triangle_input(lt, 1), 6, G, s);
    }
    for (int n = 0; n < steps && e == cudaSuccess; ++n) {
        e = launch_project(u0, G, region, s);
        if (e == cudaSuccess) e = rk4_step_patch(u0, us, k, acc, w, G, region, true, 0, s, lower ? &lt : nullptr);
    }
    if (e == cudaSuccess) {
        BSSN_LAUNCH(KC_EXPORT, k_export, row_grid(region, NCOMP), kRowThreads, s, u0, leaves_out(state), G, region, L.npts);
        if (lower)
            BSSN_LAUNCH(KC_EXPORT, k_export_lower, row_grid(region, 6), kRowThreads, s, state->traceless_K,
                        state->conformal_metric, lt.delta, G, region, L.npts);
        e = cudaGetLastError();
    }
    return cuda_status(e, "bssn_rk4_step");
}

int bssn_constraints(const BssnFields* in, const int32_t shape[3], const BssnParams* params,
                     double* hamiltonian, double* momentum, double* det_gamma, double* trace_A,
                     double* gamma_condition, void* workspace, size_t workspace_bytes, void* stream) {
    if (!fields_ok(in)) return fail(BSSN_ERR_INVALID, "null field pointer");
    if (!hamiltonian || !momentum || !det_gamma || !trace_A || !gamma_condition)
        return fail(BSSN_ERR_INVALID, "null constraint output pointer");
    int st = validate_params(params);
    if (st) return st;
    RefLayout L;
    if ((st = ref_layout(shape, L))) return st;
    Geo G;
    if ((st = make_geo(params, L.S, L.org, L.P, G))) return st;
    if (!workspace || workspace_bytes < ref_workspace_values(BSSN_OP_CONSTRAINTS, L, false) * sizeof(double))
        return fail(BSSN_ERR_WORKSPACE, "workspace missing or smaller than bssn_workspace_bytes(BSSN_OP_CONSTRAINTS)");
    cudaStream_t s = (cudaStream_t)stream;
    double* u = (double*)workspace;
    RhsWork w;
    w.d1 = u + NCOMP * L.cs;
    w.der = w.d1 + 3LL * NMIX * L.cs;
    const Box region = box_of(G);
    BSSN_LAUNCH(KC_IMPORT, k_import, row_grid(region, NCOMP), kRowThreads, s, leaves_in(in), u, G, region, L.npts);
    cudaError_t e = launch_fill_periodic(u, NCOMP, G, s);
    if (e == cudaSuccess)
        e = launch_constraints(u, w, G, region, hamiltonian, momentum, det_gamma, trace_A, gamma_condition, s);
    return cuda_status(e, "bssn_constraints");
}

// ---------------- whole-array layout conversion ----------------

static Geo plain_geo(const int32_t extent[3]) {
    Geo G;
    std::memset(&G, 0, sizeof(G));
    for (int d = 0; d < 3; ++d) G.ax[d].P = extent[d];
    G.st[2] = 1;
    G.st[1] = extent[2];
    G.st[0] = (long long)extent[1] * extent[2];
    G.cs = (long long)extent[0] * extent[1] * extent[2];
    G.ninst = 1;
    G.istride = G.cs;
    return G;
}

int bssn_fields_to_components(const BssnFields* in, double* state, const int32_t extent[3], void* stream) {
    if (!fields_ok(in) || !state || !extent) return fail(BSSN_ERR_INVALID, "null pointer");
    for (int d = 0; d < 3; ++d)
        if (extent[d] < 1) return fail(BSSN_ERR_INVALID, "array extents must be positive");
    const Geo G = plain_geo(extent);
    const Box region = full_box(G);
    BSSN_LAUNCH(KC_IMPORT, k_import, row_grid(region, NCOMP), kRowThreads, (cudaStream_t)stream, leaves_in(in),
                state, G, region, region.count);
    return cuda_status(cudaGetLastError(), "bssn_fields_to_components");
}

int bssn_components_to_fields(const double* state, BssnFields* out, const int32_t extent[3], void* stream) {
    if (!fields_ok(out) || !state || !extent) return fail(BSSN_ERR_INVALID, "null pointer");
    for (int d = 0; d < 3; ++d)
        if (extent[d] < 1) return fail(BSSN_ERR_INVALID, "array extents must be positive");
    const Geo G = plain_geo(extent);
    const Box region = full_box(G);
    BSSN_LAUNCH(KC_EXPORT, k_export, row_grid(region, NCOMP), kRowThreads, (cudaStream_t)stream, state,
                leaves_out(out), G, region, region.count);
    return cuda_status(cudaGetLastError(), "bssn_components_to_fields");
}

// ---------------- resident patch layout ----------------

static int patch_geo(const BssnPatch* patch, const BssnParams* params, Geo& G) {
    if (!patch) return fail(BSSN_ERR_INVALID, "patch is null");
    if (patch->ghost < 4) return fail(BSSN_ERR_INVALID, "patch ghost width must be at least 4");
    int S[3], org[3], P[3];
    for (int d = 0; d < 3; ++d) {
        if (patch->n[d] < 1) return fail(BSSN_ERR_INVALID, "patch extents must be positive");
        S[d] = patch->n[d];
        org[d] = patch->ghost;
        P[d] = patch->n[d] + 2 * patch->ghost;
    }
    BssnParams p;
    if (params) p = *params;
    else {
        std::memset(&p, 0, sizeof(p));
        p.dx = 1.0;
        p.mad_q = 1.0;
        for (int f = 0; f < 6; ++f) p.owned_faces[f] = 1;
        for (int d = 0; d < 3; ++d) { p.owned_shape[d] = -1; p.reduced_axes[d] = -1; }
    }
    p.guard_cells = 0;
    for (int d = 0; d < 3; ++d) p.owned_shape[d] = -1;
    return make_geo(&p, S, org, P, G);
}

// A batch: ninst instances of one patch, laid out [component][instance][padded block].
static int batch_geo(const BssnPatch* patch, int32_t ninst, const BssnParams* params, Geo& G) {
    if (ninst < 1) return fail(BSSN_ERR_INVALID, "instance count must be positive");
    const int st = patch_geo(patch, params, G);
    if (st) return st;
    G.ninst = ninst;
    G.istride = G.cs;
    G.cs *= ninst;
    return BSSN_OK;
}

static size_t patch_block(const BssnPatch* patch) {
    size_t cs = 1;
    for (int d = 0; d < 3; ++d) cs *= (size_t)(patch->n[d] + 2 * patch->ghost);
    return cs;
}

size_t bssn_batch_values(const BssnPatch* patch, int32_t ninst) {
    if (!patch || ninst < 1) return 0;
    return (size_t)NCOMP * (size_t)ninst * patch_block(patch);
}

size_t bssn_batch_workspace_bytes(const BssnPatch* patch, int32_t ninst, const BssnParams* params) {
    if (!patch || ninst < 1) return 0;
    const bool with_mom = params && params->kappa != 0.0;
    return (3 * NCOMP + rhs_work_blocks(with_mom)) * (size_t)ninst * patch_block(patch) * sizeof(double);
}

static int instance_ok(int32_t ninst, int32_t instance) {
    if (ninst < 1 || instance < 0 || instance >= ninst)
        return fail(BSSN_ERR_INVALID, "instance index outside [0, instance count)");
    return BSSN_OK;
}

int bssn_batch_import(const BssnFields* in, double* states, const BssnPatch* patch, int32_t ninst, int32_t instance,
                      void* stream) {
    if (!fields_ok(in) || !states) return fail(BSSN_ERR_INVALID, "null pointer");
    int st = instance_ok(ninst, instance);
    if (st) return st;
    Geo G;
    if ((st = batch_geo(patch, ninst, nullptr, G))) return st;
    const Box region = box_of(G);
    BSSN_LAUNCH(KC_IMPORT, k_import, row_grid(region, NCOMP), kRowThreads, (cudaStream_t)stream, leaves_in(in),
                states + (long long)instance * G.istride, G, region, region.count);
    return cuda_status(cudaGetLastError(), "bssn_batch_import");
}

int bssn_batch_export(const double* states, BssnFields* out, const BssnPatch* patch, int32_t ninst,
                      int32_t instance, void* stream) {
    if (!fields_ok(out) || !states) return fail(BSSN_ERR_INVALID, "null pointer");
    int st = instance_ok(ninst, instance);
    if (st) return st;
    Geo G;
    if ((st = batch_geo(patch, ninst, nullptr, G))) return st;
    const Box region = box_of(G);
    BSSN_LAUNCH(KC_EXPORT, k_export, row_grid(region, NCOMP), kRowThreads, (cudaStream_t)stream,
                states + (long long)instance * G.istride, leaves_out(out), G, region, region.count);
    return cuda_status(cudaGetLastError(), "bssn_batch_export");
}

int bssn_batch_fill_periodic(double* states, const BssnPatch* patch, int32_t ninst, void* stream) {
    if (!states) return fail(BSSN_ERR_INVALID, "null pointer");
    Geo G;
    const int st = batch_geo(patch, ninst, nullptr, G);
    if (st) return st;
    return cuda_status(launch_fill_periodic(states, NCOMP, G, (cudaStream_t)stream), "bssn_batch_fill_periodic");
}

int bssn_batch_rk4(double* states, const BssnPatch* patch, int32_t ninst, const BssnParams* params, int32_t steps,
                   void* workspace, size_t workspace_bytes, void* stream) {
    if (!states) return fail(BSSN_ERR_INVALID, "null pointer");
    if (steps < 0) return fail(BSSN_ERR_INVALID, "steps must be non-negative");
    int st = validate_params(params);
    if (st) return st;
    Geo G;
    if ((st = batch_geo(patch, ninst, params, G))) return st;
    const bool with_mom = params->kappa != 0.0;
    if (!workspace || workspace_bytes < bssn_batch_workspace_bytes(patch, ninst, params))
        return fail(BSSN_ERR_WORKSPACE, "workspace missing or smaller than bssn_batch_workspace_bytes");
    cudaStream_t s = (cudaStream_t)stream;
    double* us = (double*)workspace;
    double* k = us + NCOMP * G.cs;
    double* acc = k + NCOMP * G.cs;
    RhsWork w = carve_rhs_work(acc + NCOMP * G.cs, G.cs, with_mom);
    const Box region = box_of(G);
    cudaError_t e = cudaSuccess;
    for (int n = 0; n < steps && e == cudaSuccess; ++n) {
        e = launch_project(states, G, region, s);
        if (e == cudaSuccess) e = rk4_step_patch(states, us, k, acc, w, G, region, true, 0, s);
    }
    return cuda_status(e, "bssn_batch_rk4");
}

int bssn_batch_check_finite(const double* states, const BssnPatch* patch, int32_t ninst, int32_t* device_flag,
                            void* stream) {
    if (!states || !device_flag) return fail(BSSN_ERR_INVALID, "null pointer");
    Geo G;
    const int st = batch_geo(patch, ninst, nullptr, G);
    if (st) return st;
    const Box region = box_of(G);
    BSSN_LAUNCH(KC_OTHER, k_count_nonfinite, nblocks(box_threads(G, region)), kThreads, (cudaStream_t)stream, states,
                G, region, (int*)device_flag);
    return cuda_status(cudaGetLastError(), "bssn_batch_check_finite");
}

int bssn_batch_rk4_monitored(double* states, const BssnPatch* patch, int32_t ninst, const BssnParams* params,
                             int32_t steps, int32_t check_every, int32_t* device_counter, int32_t* steps_done,
                             void* workspace, size_t workspace_bytes, void* stream) {
    if (!states || !device_counter || !steps_done) return fail(BSSN_ERR_INVALID, "null pointer");
    if (check_every < 1) return fail(BSSN_ERR_INVALID, "check_every must be positive");
    *steps_done = 0;
    Geo G;
    int st = batch_geo(patch, ninst, nullptr, G);
    if (st) return st;
    cudaStream_t s = (cudaStream_t)stream;
    const Box region = box_of(G);
    int done = 0;
    for (;;) {
        cudaError_t e = cudaMemsetAsync(device_counter, 0, sizeof(int32_t), s);
        if (e == cudaSuccess) {
            BSSN_LAUNCH(KC_OTHER, k_count_nonfinite, nblocks(box_threads(G, region)), kThreads, s, states, G, region,
                        (int*)device_counter);
            e = cudaGetLastError();
        }
        int32_t count = 0;
        if (e == cudaSuccess) e = cudaMemcpyAsync(&count, device_counter, sizeof(int32_t), cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) return cuda_status(e, "bssn_batch_rk4_monitored");
        if (count > 0)
            return fail(BSSN_ERR_NONFINITE, std::to_string(count) + " non-finite owned values " +
                                                (done == 0 ? std::string("in the state before step 1")
                                                           : "after step " + std::to_string(done)));
        if (done >= steps) break;
        const int chunk = std::min(check_every, steps - done);
        if ((st = bssn_batch_rk4(states, patch, ninst, params, chunk, workspace, workspace_bytes, stream)))
            return st;
        done += chunk;
        *steps_done = done;
    }
    return BSSN_OK;
}

int bssn_tune_patch(double* states, const BssnPatch* patch, int32_t ninst, const BssnParams* params, float margin,
                    void* workspace, size_t workspace_bytes, char* report, size_t report_bytes, void* stream) {
    if (!states) return fail(BSSN_ERR_INVALID, "null pointer");
    if (!(margin > 0.0f)) return fail(BSSN_ERR_INVALID, "bssn_tune_patch: margin must be positive");
    int st = validate_params(params);
    if (st) return st;
    Geo G;
    if ((st = batch_geo(patch, ninst, params, G))) return st;
    if (!workspace || workspace_bytes < bssn_batch_workspace_bytes(patch, ninst, params))
        return fail(BSSN_ERR_WORKSPACE, "workspace missing or smaller than bssn_batch_workspace_bytes");
    cudaStream_t s = (cudaStream_t)stream;
    double* k = (double*)workspace + NCOMP * G.cs;
    RhsWork w = carve_rhs_work(k + 2 * NCOMP * G.cs, G.cs, params->kappa != 0.0);
    const Box region = box_of(G);
    std::string text;
    cudaError_t e = launch_fill_periodic(states, NCOMP, G, s);
    if (e == cudaSuccess) e = tune_rhs(states, k, w, G, region, s, 5, margin, &text);
    if (e == cudaErrorStreamCaptureUnsupported)
        return fail(BSSN_ERR_INVALID, "bssn_tune_patch: the stream is being captured; tune before capturing");
    if (e == cudaSuccess && report && report_bytes > 0) {
        const size_t n = std::min(text.size(), report_bytes - 1);
        std::memcpy(report, text.data(), n);
        report[n] = '\0';
    }
    return cuda_status(e, "bssn_tune_patch");
}

int bssn_set_tma(int32_t kernels) {
    if (kernels < 0 || kernels > BSSN_TMA_ALL) return fail(BSSN_ERR_INVALID, "kernels must be a mask of BSSN_TMA_*");
    set_tma_kernels(kernels);
    return BSSN_OK;
}

int bssn_tma_status(int32_t* timeouts, int64_t* launches) {
    if (!timeouts) return fail(BSSN_ERR_INVALID, "null pointer");
    int n = 0;
    const cudaError_t e = tma_timeouts(&n);
    *timeouts = n;
    if (launches) *launches = tma_launches();
    return cuda_status(e, "bssn_tma_status");
}

// The single-patch calls are the one-instance batch.
size_t bssn_patch_values(const BssnPatch* patch) { return bssn_batch_values(patch, 1); }

size_t bssn_patch_workspace_bytes(const BssnPatch* patch, const BssnParams* params) {
    return bssn_batch_workspace_bytes(patch, 1, params);
}

int bssn_patch_import(const BssnFields* in, double* patch_state, const BssnPatch* patch, void* stream) {
    return bssn_batch_import(in, patch_state, patch, 1, 0, stream);
}

int bssn_patch_export(const double* patch_state, BssnFields* out, const BssnPatch* patch, void* stream) {
    return bssn_batch_export(patch_state, out, patch, 1, 0, stream);
}

int bssn_patch_fill_periodic(double* patch_state, const BssnPatch* patch, void* stream) {
    return bssn_batch_fill_periodic(patch_state, patch, 1, stream);
}

int bssn_patch_rk4(double* patch_state, const BssnPatch* patch, const BssnParams* params, int32_t steps,
                   void* workspace, size_t workspace_bytes, void* stream) {
    return bssn_batch_rk4(patch_state, patch, 1, params, steps, workspace, workspace_bytes, stream);
}

int bssn_patch_check_finite(const double* patch_state, const BssnPatch* patch, int32_t* device_flag,
                            void* stream) {
    return bssn_batch_check_finite(patch_state, patch, 1, device_flag, stream);
}

}  // extern "C"
