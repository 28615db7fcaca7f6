// Fixed mesh refinement on one GPU: halo refresh, prolongation, injection,
// the stage-synchronous RK4 over a patch tree and composite constraint norms.
//
// Every patch lives in the working layout (21 components, padded by G = 4
// guards, owned samples at [4, 4+n)).  Algorithms follow uwplasma/JAX_BSSN for
// a single-tile topology:
//   halo refresh: self-wrap + linear exterior  JAX_BSSN/parallel/evolution.py:74-92,
//                                              JAX_BSSN/parallel/communication.py:36-106
//   prolongation into the exterior shell       JAX_BSSN/fmr/transfer.py:57-142, 197-244
//   injection of coincident vertices           JAX_BSSN/fmr/transfer.py:145-171, 247-252
//   prepare / stage / RK4 / injection order    JAX_BSSN/fmr/tiled.py:146-209
//   composite point-count norms                JAX_BSSN/fmr/tiled.py:212-246,
//                                              JAX_BSSN/parallel/evolution.py:145-170
// The six-node interpolation is separable and is evaluated in the
// reference's order -- along x for each of the 6x6 (y, z) source lines, then
// along y, then z -- with every product and sum rounded (no FMA), using
// weights computed on the host by the reference's product formula.
#include <array>
#include <cmath>
#include <cstring>
#include <map>
#include <vector>

#include "../../include/bssn_gb300.h"
#include "bssn_driver.h"
#include "bssn_fields.cuh"
#include "bssn_kernels.h"
#include "bssn_profile.h"

namespace bssn {

constexpr int kFmrGuard = 4;
static_assert(kFmrGuard % 2 == 0, "prolongation pairs child z samples by the parity of (z - guard)");
constexpr int kFmrThreads = 256;
static inline unsigned fmr_blocks(long long n) { return (unsigned)((n + kFmrThreads - 1) / kFmrThreads); }

struct PatchDims {
    int n[3];   // owned samples
    int P[3];   // padded extent n + 8
    long long cs;
    __host__ __device__ long long at(int x, int y, int z) const {
        return ((long long)x * P[1] + y) * P[2] + z;
    }
};

static PatchDims dims_of(const int32_t n[3]) {
    PatchDims d;
    d.cs = 1;
    for (int a = 0; a < 3; ++a) {
        d.n[a] = n[a];
        d.P[a] = n[a] + 2 * kFmrGuard;
        d.cs *= d.P[a];
    }
    return d;
}

// ---------------------------------------------------------------------------
// halo refresh along one axis (communication.py:39-106): guards take the
// periodic image of owned samples; on a Sommerfeld face they take the linear
// extrapolation base + (i - boundary) * slope instead.
// ---------------------------------------------------------------------------
__global__ void k_fmr_sweep(double* __restrict__ u, PatchDims D, int axis, int lcode, int rcode) {
    const int g = kFmrGuard;
    const int other0 = axis == 0 ? 1 : 0, other1 = axis == 2 ? 1 : 2;
    const long long slab = (long long)(2 * g) * D.P[other0] * D.P[other1];
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= slab * NCOMP) return;
    const int comp = (int)(t / slab);
    long long r = t - (long long)comp * slab;
    const int jg = (int)(r / ((long long)D.P[other0] * D.P[other1]));
    r -= (long long)jg * D.P[other0] * D.P[other1];
    const int a0 = (int)(r / D.P[other1]);
    const int a1 = (int)(r - (long long)a0 * D.P[other1]);
    const bool upper = jg >= g;
    const int i = upper ? g + D.n[axis] + (jg - g) : jg;
    int ix[3];
    ix[axis] = i;
    ix[other0] = a0;
    ix[other1] = a1;
    double* f = u + (long long)comp * D.cs;
    const int code = upper ? rcode : lcode;
    double value;
    if (code == kSommerfeld) {
        const int boundary = upper ? g + D.n[axis] - 1 : g;
        const int inward = upper ? boundary - 1 : boundary + 1;
        int jb[3] = {ix[0], ix[1], ix[2]}, jn[3] = {ix[0], ix[1], ix[2]};
        jb[axis] = boundary;
        jn[axis] = inward;
        const double base = f[D.at(jb[0], jb[1], jb[2])];
        const double nb = f[D.at(jn[0], jn[1], jn[2])];
        const double slope = upper ? __dadd_rn(base, -nb) : __dadd_rn(nb, -base);
        value = __dadd_rn(base, __dmul_rn((double)(i - boundary), slope));
    } else {
        int rel = (i - g) % D.n[axis];
        if (rel < 0) rel += D.n[axis];
        int js[3] = {ix[0], ix[1], ix[2]};
        js[axis] = g + rel;
        value = f[D.at(js[0], js[1], js[2])];
    }
    f[D.at(ix[0], ix[1], ix[2])] = value;
}

cudaError_t launch_fmr_refresh(double* u, const PatchDims& D, const int codes[6], cudaStream_t s) {
    for (int axis = 0; axis < 3; ++axis) {
        const int o0 = axis == 0 ? 1 : 0, o1 = axis == 2 ? 1 : 2;
        const long long count = (long long)(2 * kFmrGuard) * D.P[o0] * D.P[o1] * NCOMP;
        BSSN_LAUNCH(KC_TRANSFER, k_fmr_sweep, fmr_blocks(count), kFmrThreads, s, u, D, axis, codes[2 * axis],
                    codes[2 * axis + 1]);
    }
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// prolongation of the child's exterior shell (transfer.py:114-142, 205-244)
// ---------------------------------------------------------------------------
struct ProlongWeights {
    double w[2][6];  // [0]: target on a parent vertex, [1]: half-way target
};

// Six-node Lagrange weights at a target with fractional part `frac` relative
// to the node floor(t): the reference's product formula (transfer.py:57-69).
static void lagrange6(double frac, double (&w)[6]) {
    for (int k = 0; k < 6; ++k) {
        double c = 1.0;
        for (int m = 0; m < 6; ++m) {
            if (m == k) continue;
            const double t_minus_m = (2.0 + frac) - (double)m;       // t - node_m, nodes floor(t)-2+m
            c = c * (t_minus_m / ((double)k - (double)m));
        }
        w[k] = c;
    }
}

// Shell enumeration.  The child's guard shell is three dense slabs of
// (x, y, z-pair) work items (one component per grid z slice): X = guard x planes (all y, all pairs), Y =
// interior x with guard y (all pairs), Z = interior x and y with the guard
// pairs only.  Within a slab, x and y are enumerated evens first, then odds,
// and pairs fastest, so a warp shares one (x parity, y parity) class and every
// lane has work: on a part whose FP64 pipe issues two lanes per clock per SM,
// idle or divergent lanes cost as much as busy ones.
struct AxisSet {
    int lo0, hi0, lo1, hi1;   // [lo0, hi0) U [lo1, hi1)
};

__device__ __forceinline__ int parity_count(int a, int b, int f) {  // #v in [a, b), v % 2 == f
    if (b <= a) return 0;
    return ((b + 1 - f) >> 1) - ((a + 1 - f) >> 1);
}

__device__ __forceinline__ int set_count(const AxisSet& S) { return (S.hi0 - S.lo0) + (S.hi1 - S.lo1); }

// k-th element of S in the order: even elements ascending, then odd ones
__device__ __forceinline__ int set_pick(const AxisSet& S, int k) {
#pragma unroll
    for (int f = 0; f < 2; ++f) {
        const int c0 = parity_count(S.lo0, S.hi0, f), c1 = parity_count(S.lo1, S.hi1, f);
        if (k < c0) return S.lo0 + ((S.lo0 ^ f) & 1) + 2 * k;
        k -= c0;
        if (k < c1) return S.lo1 + ((S.lo1 ^ f) & 1) + 2 * k;
        k -= c1;
    }
    return -1;
}

struct ShellSlabs {
    AxisSet x[3], y[3];
    int pair_lo[3][2], pair_n[3][2];   // pair ranges [lo, lo + n) (two per slab)
    long long count[3];
};

// With g = 4 even, a child sample's parity along an axis decides its parent
// target: even samples sit on a parent node (frac 0), odd ones half-way (frac
// 1).  The six-node weights at frac 0 are exactly (0, 0, 1, 0, 0, 0), so the
// reference's sum there equals the node value (up to the sign of a zero
// result, and except that a non-finite neighbour would make the reference's
// sum NaN); such axes are skipped.  An even/odd z pair shares the same six z
// nodes (the even sample is node 2), so both come from one set of
// y-interpolated lines.  Every remaining sum runs x, then y, then z over the
// nodes in order with round-to-nearest operations, as the reference's
// separable application does.
__global__ void k_fmr_prolong(const double* __restrict__ parent, PatchDims Dp, double* __restrict__ child,
                              PatchDims Dc, int lo0, int lo1, int lo2, ProlongWeights W, ShellSlabs S) {
    const int slab = blockIdx.y;
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= S.count[slab]) return;
    const int np0 = S.pair_n[slab][0], npairs = np0 + S.pair_n[slab][1];
    const int ny = set_count(S.y[slab]);
    const long long row = t / npairs;
    const int k = (int)(t - row * npairs);
    const int x = set_pick(S.x[slab], (int)(row / ny));
    const int y = set_pick(S.y[slab], (int)(row - (row / ny) * ny));
    const int pr = k < np0 ? S.pair_lo[slab][0] + k : S.pair_lo[slab][1] + (k - np0);
    const int z0 = 2 * pr, z1 = z0 + 1;
    const int g = kFmrGuard;
    const bool xy_shell = x < g || x >= g + Dc.n[0] || y < g || y >= g + Dc.n[1];
    const bool s0 = xy_shell || z0 < g || z0 >= g + Dc.n[2];
    const bool s1 = z1 < Dc.P[2] && (xy_shell || z1 < g || z1 >= g + Dc.n[2]);
    if (!s0 && !s1) return;
    const int lo[3] = {lo0, lo1, lo2};
    const int ix[3] = {x, y, z0};
    int node0[3], frac[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        // parent padded target = lo + (ix - g)/2 + g; floor and parity
        const int twice = 2 * (lo[a] + g) + (ix[a] - g);   // 2 * target
        const int fl = twice >= 0 ? twice / 2 : -((-twice + 1) / 2);
        frac[a] = twice - 2 * fl;                          // 0 or 1 (0 for z0)
        node0[a] = fl - 2;
    }
    double w[6];
#pragma unroll
    for (int k = 0; k < 6; ++k) w[k] = W.w[1][k];
    const long long sx = (long long)Dp.P[1] * Dp.P[2];
    const bool fx = frac[0] != 0, fy = frac[1] != 0;
    {
        const int c = blockIdx.z;   // one component per grid z slice
        const double* f = parent + (long long)c * Dp.cs;
        // x-interpolated value at parent (py, pz)
        auto xval = [&](int py, int pz) -> double {
            const double* row = f + Dp.at(node0[0], py, pz);
            if (!fx) return row[2 * sx];
            double v = __dmul_rn(row[0], w[0]);
#pragma unroll
            for (int k = 1; k < 6; ++k) v = __dadd_rn(v, __dmul_rn(row[k * sx], w[k]));
            return v;
        };
        // x- then y-interpolated value at parent z index pz
        auto yval = [&](int pz) -> double {
            if (!fy) return xval(node0[1] + 2, pz);
            double v = __dmul_rn(xval(node0[1], pz), w[0]);
#pragma unroll 1
            for (int k = 1; k < 6; ++k) v = __dadd_rn(v, __dmul_rn(xval(node0[1] + k, pz), w[k]));
            return v;
        };
        if (s1) {
            double line[6];
#pragma unroll
            for (int k = 0; k < 6; ++k) line[k] = yval(node0[2] + k);
            if (s0) child[(long long)c * Dc.cs + Dc.at(x, y, z0)] = line[2];
            double acc = __dmul_rn(line[0], w[0]);
#pragma unroll
            for (int k = 1; k < 6; ++k) acc = __dadd_rn(acc, __dmul_rn(line[k], w[k]));
            child[(long long)c * Dc.cs + Dc.at(x, y, z1)] = acc;
        } else {
            child[(long long)c * Dc.cs + Dc.at(x, y, z0)] = yval(node0[2] + 2);
        }
    }
}

static ProlongWeights prolong_weights() {
    ProlongWeights W;
    lagrange6(0.0, W.w[0]);
    lagrange6(0.5, W.w[1]);
    return W;
}

static AxisSet guard_set(int n, int g) { return AxisSet{0, g, g + n, n + 2 * g}; }
static AxisSet interior_set(int n, int g) { return AxisSet{g, g + n, 0, 0}; }
static AxisSet full_set(int n, int g) { return AxisSet{0, n + 2 * g, 0, 0}; }

static ShellSlabs shell_slabs(const PatchDims& Dc) {
    const int g = kFmrGuard;
    const int pairs = (Dc.P[2] + 1) / 2;
    // pairs holding a guard z sample: z < g (pairs [0, g/2)) and z >= g + n
    const int hi_first = (g + Dc.n[2] - 1) / 2;   // first pair whose odd member reaches the upper guard
    ShellSlabs S;
    S.x[0] = guard_set(Dc.n[0], g);    S.y[0] = full_set(Dc.n[1], g);
    S.x[1] = interior_set(Dc.n[0], g); S.y[1] = guard_set(Dc.n[1], g);
    S.x[2] = interior_set(Dc.n[0], g); S.y[2] = interior_set(Dc.n[1], g);
    for (int k = 0; k < 2; ++k) {
        S.pair_lo[k][0] = 0; S.pair_n[k][0] = pairs;
        S.pair_lo[k][1] = 0; S.pair_n[k][1] = 0;
    }
    S.pair_lo[2][0] = 0;        S.pair_n[2][0] = g / 2;
    S.pair_lo[2][1] = hi_first; S.pair_n[2][1] = pairs - hi_first;
    for (int k = 0; k < 3; ++k) {
        const long long nx = (S.x[k].hi0 - S.x[k].lo0) + (S.x[k].hi1 - S.x[k].lo1);
        const long long ny = (S.y[k].hi0 - S.y[k].lo0) + (S.y[k].hi1 - S.y[k].lo1);
        S.count[k] = nx * ny * (S.pair_n[k][0] + S.pair_n[k][1]);
    }
    return S;
}

cudaError_t launch_fmr_prolong(const double* parent, const PatchDims& Dp, double* child, const PatchDims& Dc,
                               const int lo[3], cudaStream_t s) {
    const ShellSlabs S = shell_slabs(Dc);
    long long most = 0;
    for (int k = 0; k < 3; ++k) most = S.count[k] > most ? S.count[k] : most;
    const dim3 grid(fmr_blocks(most), 3, NCOMP);
    BSSN_LAUNCH(KC_TRANSFER, k_fmr_prolong, grid, kFmrThreads, s, parent, Dp, child, Dc, lo[0], lo[1], lo[2],
                prolong_weights(), S);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// FP32 form: the same prolongation in float on perturbations.  Interpolation
// is linear with weights summing to one, so interpolating u - b and adding b
// back gives the interpolant of u for any constant b.  The parent window the
// child's stencils reach is converted once to float perturbations about each
// component's value at the window's first sample (a uniform shift or any
// other offset drops out), interpolated in float, and written to the FP64
// child guards as b + result.  Node shortcuts and enumeration as above.
// ---------------------------------------------------------------------------
struct Window {
    int lo[3], n[3];
    long long cs;   // samples per component block
    __host__ __device__ long long at(int x, int y, int z) const {
        return ((long long)(x - lo[0]) * n[1] + (y - lo[1])) * n[2] + (z - lo[2]);
    }
};

__global__ void k_fmr_window_f32(const double* __restrict__ parent, PatchDims Dp, Window Wn, float* __restrict__ out) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const int c = blockIdx.y;
    if (t >= Wn.cs) return;
    const int x = Wn.lo[0] + (int)(t / ((long long)Wn.n[1] * Wn.n[2]));
    const long long r = t % ((long long)Wn.n[1] * Wn.n[2]);
    const int y = Wn.lo[1] + (int)(r / Wn.n[2]);
    const int z = Wn.lo[2] + (int)(r % Wn.n[2]);
    const double* f = parent + (long long)c * Dp.cs;
    const double b = f[Dp.at(Wn.lo[0], Wn.lo[1], Wn.lo[2])];
    out[(long long)c * Wn.cs + t] = static_cast<float>(f[Dp.at(x, y, z)] - b);
}

__global__ void __launch_bounds__(kFmrThreads, 4)
k_fmr_prolong_f32(const double* __restrict__ parent, PatchDims Dp, const float* __restrict__ win,
                                  Window Wn, double* __restrict__ child, PatchDims Dc, int lo0, int lo1, int lo2,
                                  ProlongWeights W, ShellSlabs S) {
    const int slab = blockIdx.y;
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= S.count[slab]) return;
    const int np0 = S.pair_n[slab][0], npairs = np0 + S.pair_n[slab][1];
    const int ny = set_count(S.y[slab]);
    const long long row = t / npairs;
    const int k = (int)(t - row * npairs);
    const int x = set_pick(S.x[slab], (int)(row / ny));
    const int y = set_pick(S.y[slab], (int)(row - (row / ny) * ny));
    const int pr = k < np0 ? S.pair_lo[slab][0] + k : S.pair_lo[slab][1] + (k - np0);
    const int z0 = 2 * pr, z1 = z0 + 1;
    const int g = kFmrGuard;
    const bool xy_shell = x < g || x >= g + Dc.n[0] || y < g || y >= g + Dc.n[1];
    const bool s0 = xy_shell || z0 < g || z0 >= g + Dc.n[2];
    const bool s1 = z1 < Dc.P[2] && (xy_shell || z1 < g || z1 >= g + Dc.n[2]);
    if (!s0 && !s1) return;
    const int lo[3] = {lo0, lo1, lo2};
    const int ix[3] = {x, y, z0};
    int node0[3], frac[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const int twice = 2 * (lo[a] + g) + (ix[a] - g);
        const int fl = twice >= 0 ? twice / 2 : -((-twice + 1) / 2);
        frac[a] = twice - 2 * fl;
        node0[a] = fl - 2;
    }
    float w[6];
#pragma unroll
    for (int q = 0; q < 6; ++q) w[q] = static_cast<float>(W.w[1][q]);
    const long long sx = (long long)Wn.n[1] * Wn.n[2];
    const bool fx = frac[0] != 0, fy = frac[1] != 0;
    const int c = blockIdx.z;
    const float* f = win + (long long)c * Wn.cs;
    const double b = parent[(long long)c * Dp.cs + Dp.at(Wn.lo[0], Wn.lo[1], Wn.lo[2])];
    auto xval = [&](int py, int pz) -> float {
        const float* rowp = f + Wn.at(node0[0], py, pz);
        if (!fx) return rowp[2 * sx];
        float v = rowp[0] * w[0];
#pragma unroll
        for (int q = 1; q < 6; ++q) v += rowp[q * sx] * w[q];
        return v;
    };
    auto yval = [&](int pz) -> float {
        if (!fy) return xval(node0[1] + 2, pz);
        float v = xval(node0[1], pz) * w[0];
#pragma unroll
        for (int q = 1; q < 6; ++q) v += xval(node0[1] + q, pz) * w[q];
        return v;
    };
    double* out = child + (long long)c * Dc.cs;
    if (s1) {
        float line[6];
#pragma unroll
        for (int q = 0; q < 6; ++q) line[q] = yval(node0[2] + q);
        if (s0) out[Dc.at(x, y, z0)] = b + static_cast<double>(line[2]);
        float acc = line[0] * w[0];
#pragma unroll
        for (int q = 1; q < 6; ++q) acc += line[q] * w[q];
        out[Dc.at(x, y, z1)] = b + static_cast<double>(acc);
    } else {
        out[Dc.at(x, y, z0)] = b + static_cast<double>(yval(node0[2] + 2));
    }
}

// The parent samples the child's guard shell reaches: six nodes around every
// target lo + (i - g)/2 + g, i over the child's padded extent.  A child
// strictly inside its parent keeps the window inside the parent's padded
// array; `ok` is false otherwise or when the window outgrows the child's
// float scratch, and the caller then takes the FP64 prolongation.
static Window prolong_window(const PatchDims& Dp, const PatchDims& Dc, const int lo[3], bool& ok) {
    const int g = kFmrGuard;
    auto floor_half = [](int twice) { return twice >= 0 ? twice / 2 : -((-twice + 1) / 2); };
    Window Wn;
    Wn.cs = 1;
    ok = true;
    for (int a = 0; a < 3; ++a) {
        const int first = floor_half(2 * (lo[a] + g) + (0 - g)) - 2;
        const int last = floor_half(2 * (lo[a] + g) + (Dc.P[a] - 1 - g)) + 3;
        ok = ok && first >= 0 && last <= Dp.P[a] - 1;
        Wn.lo[a] = first;
        Wn.n[a] = last - first + 1;
        Wn.cs *= Wn.n[a];
    }
    ok = ok && Wn.cs <= Dc.cs;
    return Wn;
}

// FP32-form prolongation; `scratch` holds NCOMP * Dc.cs floats.
cudaError_t launch_fmr_prolong_f32(const double* parent, const PatchDims& Dp, double* child, const PatchDims& Dc,
                                   const int lo[3], float* scratch, cudaStream_t s) {
    bool ok = false;
    const Window Wn = prolong_window(Dp, Dc, lo, ok);
    if (!ok) return launch_fmr_prolong(parent, Dp, child, Dc, lo, s);
    BSSN_LAUNCH(KC_TRANSFER, k_fmr_window_f32, dim3(fmr_blocks(Wn.cs), NCOMP), kFmrThreads, s, parent, Dp, Wn,
                scratch);
    const ShellSlabs S = shell_slabs(Dc);
    long long most = 0;
    for (int k = 0; k < 3; ++k) most = S.count[k] > most ? S.count[k] : most;
    const dim3 grid(fmr_blocks(most), 3, NCOMP);
    BSSN_LAUNCH(KC_TRANSFER, k_fmr_prolong_f32, grid, kFmrThreads, s, parent, Dp, scratch, Wn, child, Dc, lo[0],
                lo[1], lo[2], prolong_weights(), S);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// injection of coincident owned fine vertices (transfer.py:145-171)
// ---------------------------------------------------------------------------
__global__ void k_fmr_inject(double* __restrict__ parent, PatchDims Dp, const double* __restrict__ child,
                             PatchDims Dc, int lo0, int lo1, int lo2) {
    const int m0 = (Dc.n[0] + 1) / 2, m1 = (Dc.n[1] + 1) / 2, m2 = (Dc.n[2] + 1) / 2;
    const long long count = (long long)m0 * m1 * m2;
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= count * NCOMP) return;
    const int c = (int)(t / count);
    long long r = t - (long long)c * count;
    const int a = (int)(r / ((long long)m1 * m2));
    r -= (long long)a * m1 * m2;
    const int b = (int)(r / m2);
    const int e = (int)(r - (long long)b * m2);
    const int g = kFmrGuard;
    const double v = child[(long long)c * Dc.cs + Dc.at(g + 2 * a, g + 2 * b, g + 2 * e)];
    parent[(long long)c * Dp.cs + Dp.at(g + lo0 + a, g + lo1 + b, g + lo2 + e)] = v;
}

cudaError_t launch_fmr_inject(double* parent, const PatchDims& Dp, const double* child, const PatchDims& Dc,
                              const int lo[3], cudaStream_t s) {
    const long long count = (long long)((Dc.n[0] + 1) / 2) * ((Dc.n[1] + 1) / 2) * ((Dc.n[2] + 1) / 2) * NCOMP;
    BSSN_LAUNCH(KC_TRANSFER, k_fmr_inject, fmr_blocks(count), kFmrThreads, s, parent, Dp, child, Dc, lo[0], lo[1],
                lo[2]);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// masked point-count statistics of the constraint fields (deterministic):
// per constraint (H, M, det-1, trA, Gamma) the sum of squares and max |.| over
// owned samples not covered by a child; block partials in a fixed order, then
// one block folds them.
// ---------------------------------------------------------------------------
struct CoverBoxes {
    int count;
    int lo[8][3], hi[8][3];  // inclusive, in owned (active) indices
};

constexpr int kStatThreads = 256;
constexpr int kStatBlocks = 304;

__device__ __forceinline__ bool covered(const CoverBoxes& C, int x, int y, int z) {
    for (int b = 0; b < C.count; ++b)
        if (x >= C.lo[b][0] && x <= C.hi[b][0] && y >= C.lo[b][1] && y <= C.hi[b][1] && z >= C.lo[b][2] &&
            z <= C.hi[b][2])
            return true;
    return false;
}

// fields: 9 blocks of `npts` (H, M0, M1, M2, det, trA, G0, G1, G2) over the owned box n
__global__ void __launch_bounds__(kStatThreads)
k_stats_partial(const double* __restrict__ fields, int n0, int n1, int n2, CoverBoxes C, double* __restrict__ part) {
    const long long npts = (long long)n0 * n1 * n2;
    __shared__ double ssq[5][kStatThreads];
    __shared__ double smx[5][kStatThreads];
    double sq[5] = {0, 0, 0, 0, 0}, mx[5] = {0, 0, 0, 0, 0};
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < npts;
         t += (long long)gridDim.x * blockDim.x) {
        const int x = (int)(t / ((long long)n1 * n2));
        const long long r = t - (long long)x * n1 * n2;
        const int y = (int)(r / n2);
        const int z = (int)(r - (long long)y * n2);
        if (covered(C, x, y, z)) continue;
        const int group[9] = {0, 1, 1, 1, 2, 3, 4, 4, 4};
        for (int f = 0; f < 9; ++f) {
            const double v = fields[(long long)f * npts + t];
            sq[group[f]] += v * v;
            mx[group[f]] = fmax(mx[group[f]], fabs(v));
        }
    }
    for (int q = 0; q < 5; ++q) {
        ssq[q][threadIdx.x] = sq[q];
        smx[q][threadIdx.x] = mx[q];
    }
    __syncthreads();
    for (int stride = kStatThreads / 2; stride > 0; stride >>= 1) {
        if ((int)threadIdx.x < stride)
            for (int q = 0; q < 5; ++q) {
                ssq[q][threadIdx.x] += ssq[q][threadIdx.x + stride];
                smx[q][threadIdx.x] = fmax(smx[q][threadIdx.x], smx[q][threadIdx.x + stride]);
            }
        __syncthreads();
    }
    if (threadIdx.x == 0)
        for (int q = 0; q < 5; ++q) {
            part[blockIdx.x * 10 + 2 * q] = ssq[q][0];
            part[blockIdx.x * 10 + 2 * q + 1] = smx[q][0];
        }
}

__global__ void k_stats_fold(const double* __restrict__ part, int nparts, double* __restrict__ out) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    for (int q = 0; q < 5; ++q) {
        double s = 0.0, m = 0.0;
        for (int b = 0; b < nparts; ++b) {
            s += part[b * 10 + 2 * q];
            m = fmax(m, part[b * 10 + 2 * q + 1]);
        }
        out[2 * q] += s;
        out[2 * q + 1] = fmax(out[2 * q + 1], m);
    }
}

// ---------------------------------------------------------------------------
// patch geometry for the RHS: owned box [4, 4+n), coordinates of padded
// index 0 = origin - 4 dx (JAX_BSSN/parallel/evolution.py:19-38)
// ---------------------------------------------------------------------------
static int fmr_geo(const BssnParams* p, const PatchDims& D, Geo& G) {
    BssnParams q = *p;
    q.guard_cells = 0;
    for (int d = 0; d < 3; ++d) q.owned_shape[d] = -1;
    for (int f = 0; f < 6; ++f) q.owned_faces[f] = 1;
    int S[3], org[3], P[3];
    for (int d = 0; d < 3; ++d) {
        S[d] = D.n[d];
        org[d] = kFmrGuard;
        P[d] = D.P[d];
    }
    const int st = make_geo(&q, S, org, P, G);
    if (st) return st;
    for (int d = 0; d < 3; ++d) {
        // the reference's tile-local minimum: origin + (0 - guard) * dx
        G.ax[d].xmin = p->xmin[d] + (double)(0 - kFmrGuard) * p->dx;
        G.ax[d].org = 0;
    }
    return BSSN_OK;
}

}  // namespace bssn

using namespace bssn;

namespace {

struct FmrPlan {
    int npatch;
    std::vector<PatchDims> dims;
    std::vector<Geo> geo;
    std::vector<int> parent;
    std::vector<std::array<int, 3>> lo, hi;
    std::vector<std::array<int, 6>> codes;
    bool with_mom = false;
};

int make_plan(const BssnFmrPatch* patches, const BssnParams* params, int32_t npatch, FmrPlan& plan) {
    if (!patches || !params || npatch < 1) return fail(BSSN_ERR_INVALID, "FMR needs at least one patch");
    if (npatch > 64) return fail(BSSN_ERR_INVALID, "FMR supports at most 64 patches");
    plan.npatch = npatch;
    for (int p = 0; p < npatch; ++p) {
        int st = validate_params(&params[p]);
        if (st) return st;
        const BssnFmrPatch& P = patches[p];
        for (int a = 0; a < 3; ++a)
            if (P.n[a] < 1) return fail(BSSN_ERR_INVALID, "FMR patch extents must be positive");
        PatchDims D = dims_of(P.n);
        Geo G;
        if ((st = fmr_geo(&params[p], D, G))) return st;
        plan.dims.push_back(D);
        plan.geo.push_back(G);
        plan.parent.push_back(p == 0 ? -1 : P.parent);
        std::array<int, 3> lo{P.coarse_lo[0], P.coarse_lo[1], P.coarse_lo[2]};
        std::array<int, 3> hi{P.coarse_hi[0], P.coarse_hi[1], P.coarse_hi[2]};
        plan.lo.push_back(lo);
        plan.hi.push_back(hi);
        std::array<int, 6> c;
        for (int f = 0; f < 6; ++f) c[f] = params[p].bc[f];
        plan.codes.push_back(c);
        plan.with_mom = plan.with_mom || params[p].kappa != 0.0;
        if (p == 0) continue;
        if (P.parent < 0 || P.parent >= p) return fail(BSSN_ERR_INVALID, "FMR patches must follow their parent");
        const PatchDims& Dp = plan.dims[P.parent];
        for (int a = 0; a < 3; ++a) {
            if (lo[a] <= 0 || hi[a] >= Dp.n[a] - 1 || hi[a] < lo[a])
                return fail(BSSN_ERR_INVALID, "every child patch must be strictly inside its parent");
            if (P.n[a] != 2 * (hi[a] - lo[a]) + 1)
                return fail(BSSN_ERR_INVALID, "FMR child active shape does not match its parent bounds");
        }
    }
    return BSSN_OK;
}

size_t patch_work_values(const PatchDims& D, bool with_mom) {
    return (3 * NCOMP + rhs_work_blocks(with_mom)) * (size_t)D.cs;
}

struct PatchWork {
    double* us;
    double* k;
    double* acc;
    RhsWork rw;
};

std::vector<PatchWork> carve(const FmrPlan& plan, double* base) {
    std::vector<PatchWork> out;
    for (int p = 0; p < plan.npatch; ++p) {
        const long long cs = plan.dims[p].cs;
        PatchWork w;
        w.us = base;
        w.k = base + NCOMP * cs;
        w.acc = base + 2 * NCOMP * cs;
        w.rw = carve_rhs_work(base + 3 * NCOMP * cs, cs, plan.with_mom);
        out.push_back(w);
        base += patch_work_values(plan.dims[p], plan.with_mom);
    }
    return out;
}

Box owned_box(const Geo& G) { return box_of(G); }

// Prolongation into child p: the bitwise FP64 form, or (FP32 form, with the
// patch work available) the float form using the child's float RHS scratch,
// which is free between RHS evaluations.
cudaError_t prolong_child(const FmrPlan& plan, double* const* u, int p, const std::vector<PatchWork>* w,
                          cudaStream_t s) {
    const int q = plan.parent[p];
    if (w && float_form(plan.geo[p].precision))
        return launch_fmr_prolong_f32(u[q], plan.dims[q], u[p], plan.dims[p], plan.lo[p].data(), (*w)[p].rw.uf, s);
    return launch_fmr_prolong(u[q], plan.dims[q], u[p], plan.dims[p], plan.lo[p].data(), s);
}

// prepare: (project owned), refresh, prolong from the prepared parent -- parent first
cudaError_t prepare(const FmrPlan& plan, double* const* u, bool project, cudaStream_t s,
                    const std::vector<PatchWork>* w = nullptr) {
    cudaError_t e = cudaSuccess;
    for (int p = 0; p < plan.npatch && e == cudaSuccess; ++p) {
        if (project) e = launch_project(u[p], plan.geo[p], owned_box(plan.geo[p]), s);
        // a child's guard shell is overwritten whole by the prolongation, so
        // only the root's guards take the halo refresh
        if (e == cudaSuccess && p == 0) e = launch_fmr_refresh(u[p], plan.dims[p], plan.codes[p].data(), s);
        if (e == cudaSuccess && p > 0) e = prolong_child(plan, u, p, w, s);
    }
    return e;
}

// Streams for the children's stage work (per device and host thread), so
// that every patch's RHS and stage combination run concurrently: they touch
// only their own patch.  Profiling and calls captured before the streams exist
// run serially on the caller's stream.
struct PatchStreams {
    std::vector<cudaStream_t> s;
    std::vector<cudaEvent_t> join;
    cudaEvent_t fork = nullptr;
};

PatchStreams* patch_streams(int n, cudaStream_t caller) {
    if (n <= 0 || profiling_enabled()) return nullptr;
    thread_local std::map<int, PatchStreams> all;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    PatchStreams& P = all[dev];
    if ((int)P.s.size() >= n && P.fork) return &P;
    cudaStreamCaptureStatus status = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(caller, &status) != cudaSuccess || status != cudaStreamCaptureStatusNone) {
        cudaGetLastError();
        return nullptr;
    }
    if (!P.fork && cudaEventCreateWithFlags(&P.fork, cudaEventDisableTiming) != cudaSuccess) {
        cudaGetLastError();
        P.fork = nullptr;
        return nullptr;
    }
    while ((int)P.s.size() < n) {
        cudaStream_t st = nullptr;
        cudaEvent_t ev = nullptr;
        if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess ||
            cudaEventCreateWithFlags(&ev, cudaEventDisableTiming) != cudaSuccess) {
            cudaGetLastError();
            return nullptr;
        }
        P.s.push_back(st);
        P.join.push_back(ev);
    }
    return &P;
}

cudaError_t fmr_step(const FmrPlan& plan, double* const* u, const std::vector<PatchWork>& w, double dt,
                     cudaStream_t s) {
    const int np = plan.npatch;
    std::vector<double*> us(np);
    for (int p = 0; p < np; ++p) us[p] = w[p].us;
    PatchStreams* PS = patch_streams(np - 1, s);
    cudaError_t e = prepare(plan, u, true, s, &w);  // s0
    for (int stage = 1; stage <= 4 && e == cudaSuccess; ++stage) {
        double* const* src = stage == 1 ? u : us.data();
        if (PS) {
            cudaEventRecord(PS->fork, s);
            for (int p = 1; p < np; ++p) cudaStreamWaitEvent(PS->s[p - 1], PS->fork, 0);
        }
        // each patch's RHS, then its stage combination on owned samples with
        // projection (= project_owned of the next prepare), on its own stream
        for (int p = 0; p < np && e == cudaSuccess; ++p) {
            const cudaStream_t sp = (PS && p > 0) ? PS->s[p - 1] : s;
            e = launch_rhs(src[p], w[p].k, w[p].rw, plan.geo[p], owned_box(plan.geo[p]), sp);
            double* out = stage == 4 ? u[p] : us[p];
            if (e == cudaSuccess)
                e = launch_rk4_stage(u[p], w[p].k, w[p].acc, out, plan.geo[p], owned_box(plan.geo[p]), stage, dt,
                                     /*final_form=*/1, /*project=*/1, sp);
        }
        if (PS)
            for (int p = 1; p < np; ++p) {
                cudaEventRecord(PS->join[p - 1], PS->s[p - 1]);
                cudaStreamWaitEvent(s, PS->join[p - 1], 0);
            }
        if (stage < 4 && e == cudaSuccess) {
            // refresh + prolong of the next stage state (projection already applied)
            for (int p = 0; p < np && e == cudaSuccess; ++p) {
                e = p == 0 ? launch_fmr_refresh(us[p], plan.dims[p], plan.codes[p].data(), s)
                           : prolong_child(plan, us.data(), p, &w, s);
            }
        }
    }
    // injection deepest first, re-projecting each receiving parent
    for (int c = np - 1; c >= 1 && e == cudaSuccess; --c) {
        const int q = plan.parent[c];
        e = launch_fmr_inject(u[q], plan.dims[q], u[c], plan.dims[c], plan.lo[c].data(), s);
        if (e == cudaSuccess) e = launch_project(u[q], plan.geo[q], owned_box(plan.geo[q]), s);
    }
    if (e == cudaSuccess) e = prepare(plan, u, false, s, &w);
    return e;
}

}  // namespace

extern "C" {

size_t bssn_fmr_workspace_bytes(const BssnFmrPatch* patches, const BssnParams* params, int32_t npatch) {
    FmrPlan plan;
    if (make_plan(patches, params, npatch, plan) != BSSN_OK) return 0;
    size_t total = 0;
    for (int p = 0; p < npatch; ++p) total += patch_work_values(plan.dims[p], plan.with_mom);
    return total * sizeof(double);
}

int bssn_fmr_refresh(double* state, const int32_t n[3], const int32_t codes[6], void* stream) {
    if (!state || !n || !codes) return fail(BSSN_ERR_INVALID, "null pointer");
    for (int a = 0; a < 3; ++a)
        if (n[a] < 1) return fail(BSSN_ERR_INVALID, "patch extents must be positive");
    int c[6];
    for (int f = 0; f < 6; ++f) c[f] = codes[f];
    return cuda_status(launch_fmr_refresh(state, dims_of(n), c, (cudaStream_t)stream), "bssn_fmr_refresh");
}

int bssn_fmr_prolong(const double* parent, const int32_t parent_n[3], double* child, const int32_t child_n[3],
                     const int32_t coarse_lo[3], void* stream) {
    if (!parent || !child || !parent_n || !child_n || !coarse_lo) return fail(BSSN_ERR_INVALID, "null pointer");
    for (int a = 0; a < 3; ++a) {
        const int hi = coarse_lo[a] + (child_n[a] - 1) / 2;
        if (child_n[a] < 1 || (child_n[a] % 2) == 0 || coarse_lo[a] <= 0 || hi >= parent_n[a] - 1)
            return fail(BSSN_ERR_INVALID, "every child patch must be strictly inside its parent");
    }
    const int lo[3] = {coarse_lo[0], coarse_lo[1], coarse_lo[2]};
    return cuda_status(launch_fmr_prolong(parent, dims_of(parent_n), child, dims_of(child_n), lo, (cudaStream_t)stream),
                       "bssn_fmr_prolong");
}

int bssn_fmr_inject(double* parent, const int32_t parent_n[3], const double* child, const int32_t child_n[3],
                    const int32_t coarse_lo[3], void* stream) {
    if (!parent || !child || !parent_n || !child_n || !coarse_lo) return fail(BSSN_ERR_INVALID, "null pointer");
    for (int a = 0; a < 3; ++a) {
        const int hi = coarse_lo[a] + (child_n[a] - 1) / 2;
        if (child_n[a] < 1 || (child_n[a] % 2) == 0 || coarse_lo[a] < 0 || hi > parent_n[a] - 1)
            return fail(BSSN_ERR_INVALID, "child does not fit inside its parent");
    }
    const int lo[3] = {coarse_lo[0], coarse_lo[1], coarse_lo[2]};
    return cuda_status(launch_fmr_inject(parent, dims_of(parent_n), child, dims_of(child_n), lo, (cudaStream_t)stream),
                       "bssn_fmr_inject");
}

int bssn_fmr_rk4_step(double* const* states, const BssnFmrPatch* patches, const BssnParams* params,
                      int32_t npatch, int32_t steps, void* workspace, size_t workspace_bytes, void* stream) {
    if (!states) return fail(BSSN_ERR_INVALID, "null state array");
    if (steps < 0) return fail(BSSN_ERR_INVALID, "steps must be non-negative");
    FmrPlan plan;
    int st = make_plan(patches, params, npatch, plan);
    if (st) return st;
    for (int p = 0; p < npatch; ++p)
        if (!states[p]) return fail(BSSN_ERR_INVALID, "null patch state");
    const double dt = params[0].dt;
    for (int p = 1; p < npatch; ++p)
        if (std::fabs(params[p].dt - dt) > 1e-5 * std::fabs(dt) + 1e-8)
            return fail(BSSN_ERR_INVALID, "stage-synchronous FMR requires identical timesteps");
    if (!workspace || workspace_bytes < bssn_fmr_workspace_bytes(patches, params, npatch))
        return fail(BSSN_ERR_WORKSPACE, "workspace missing or smaller than bssn_fmr_workspace_bytes");
    const std::vector<PatchWork> w = carve(plan, (double*)workspace);
    cudaError_t e = cudaSuccess;
    for (int n = 0; n < steps && e == cudaSuccess; ++n) e = fmr_step(plan, states, w, dt, (cudaStream_t)stream);
    return cuda_status(e, "bssn_fmr_rk4_step");
}

int bssn_fmr_prepare(double* const* states, const BssnFmrPatch* patches, const BssnParams* params, int32_t npatch,
                     int32_t project, void* stream) {
    if (!states) return fail(BSSN_ERR_INVALID, "null state array");
    FmrPlan plan;
    int st = make_plan(patches, params, npatch, plan);
    if (st) return st;
    return cuda_status(prepare(plan, states, project != 0, (cudaStream_t)stream), "bssn_fmr_prepare");
}

int bssn_fmr_stage_rhs(double* const* states, double* const* rhs, const BssnFmrPatch* patches,
                       const BssnParams* params, int32_t npatch, void* workspace, size_t workspace_bytes,
                       void* stream) {
    if (!states || !rhs) return fail(BSSN_ERR_INVALID, "null state array");
    FmrPlan plan;
    int st = make_plan(patches, params, npatch, plan);
    if (st) return st;
    if (!workspace || workspace_bytes < bssn_fmr_workspace_bytes(patches, params, npatch))
        return fail(BSSN_ERR_WORKSPACE, "workspace missing or smaller than bssn_fmr_workspace_bytes");
    const std::vector<PatchWork> w = carve(plan, (double*)workspace);
    cudaStream_t s = (cudaStream_t)stream;
    cudaError_t e = prepare(plan, states, true, s);
    for (int p = 0; p < npatch && e == cudaSuccess; ++p)
        e = launch_rhs(states[p], rhs[p], w[p].rw, plan.geo[p], owned_box(plan.geo[p]), s);
    return cuda_status(e, "bssn_fmr_stage_rhs");
}

int bssn_fmr_constraint_stats(double* const* states, const BssnFmrPatch* patches, const BssnParams* params,
                              int32_t npatch, double* stats, void* workspace, size_t workspace_bytes,
                              void* stream) {
    if (!states || !stats) return fail(BSSN_ERR_INVALID, "null pointer");
    FmrPlan plan;
    int st = make_plan(patches, params, npatch, plan);
    if (st) return st;
    size_t need = 0;
    for (int p = 0; p < npatch; ++p) {
        const PatchDims& D = plan.dims[p];
        const size_t npts = (size_t)D.n[0] * D.n[1] * D.n[2];
        const size_t v = (3 * NMIX + 24) * (size_t)D.cs + 9 * npts + 10 * kStatBlocks;
        need = v > need ? v : need;
    }
    if (!workspace || workspace_bytes < need * sizeof(double))
        return fail(BSSN_ERR_WORKSPACE, "workspace smaller than the constraint-statistics need");
    cudaStream_t s = (cudaStream_t)stream;
    cudaError_t e = prepare(plan, states, false, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(stats, 0, 10 * sizeof(double), s);
    for (int p = 0; p < npatch && e == cudaSuccess; ++p) {
        const PatchDims& D = plan.dims[p];
        const long long npts = (long long)D.n[0] * D.n[1] * D.n[2];
        RhsWork rw;
        rw.d1 = (double*)workspace;
        rw.der = rw.d1 + 3LL * NMIX * D.cs;
        double* fields = rw.der + 24LL * D.cs;
        double* part = fields + 9 * npts;
        e = launch_constraints(states[p], rw, plan.geo[p], owned_box(plan.geo[p]), fields, fields + npts,
                               fields + 4 * npts, fields + 5 * npts, fields + 6 * npts, s);
        CoverBoxes C;
        std::memset(&C, 0, sizeof(C));
        for (int c = 1; c < npatch; ++c) {
            if (plan.parent[c] != p || C.count >= 8) continue;
            for (int a = 0; a < 3; ++a) {
                C.lo[C.count][a] = plan.lo[c][a];
                C.hi[C.count][a] = plan.hi[c][a];
            }
            ++C.count;
        }
        if (e == cudaSuccess) {
            BSSN_LAUNCH(KC_CONSTRAINTS, k_stats_partial, kStatBlocks, kStatThreads, s, fields, D.n[0], D.n[1], D.n[2],
                        C, part);
            BSSN_LAUNCH(KC_CONSTRAINTS, k_stats_fold, 1, 32, s, part, kStatBlocks, stats);
            e = cudaGetLastError();
        }
    }
    return cuda_status(e, "bssn_fmr_constraint_stats");
}

}  // extern "C"
