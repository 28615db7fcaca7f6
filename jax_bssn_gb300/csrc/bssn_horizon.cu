// Apparent-horizon finder (JAX_BSSN/utilities/apparent_horizon.py and
// hermite_interpolation.py):
//   geometry sampling    C1 Hermite interpolation of the physical metric and
//                        extrinsic curvature with fourth-order nodal slopes
//                        (hermite_interpolation.py:12-38) on a radial line, a
//                        signed x-z plane or a Cartesian volume, the tensors
//                        carried to the sample point by the radial projector or
//                        the azimuthal rotation (apparent_horizon.py:22-98);
//                        the metric's spatial derivative is the analytic
//                        derivative of the Hermite basis through the same maps
//                        (the reference takes it with jax.jacfwd, :96);
//   angular derivatives  fourth-order differences on the full (theta, phi)
//                        grid, a pole ghost being the node half a turn round
//                        the azimuth (:114-144), in the reference's order;
//   surface              the expansion D_i s^i + K_ij s^i s^j - K and the
//                        regular area density at every node (:160-236);
//   Newton Jacobian      row i of dTheta/dh from the six pointwise partials of
//                        Theta_i (in h_i, geometry resampled, and in its five
//                        angular derivatives, geometry fixed; central
//                        differences) times the difference stencils.  The
//                        reference differentiates the discrete residual with
//                        jax.linearize (:239-250) and stores it dense; here the
//                        rows land directly in band storage: with theta-major
//                        unknowns a node couples to polar rows t-2..t+2 (pole
//                        ghosts fold back onto rows 0, 1 and n-1, n-2) and to
//                        azimuthal offsets -2..2 with wrap, so |i - j| < 3 n_phi;
//   Newton solve         band LU with partial pivoting (the pivot rule of a
//                        dense getrf: first largest modulus in the column), the
//                        right-hand side carried as an extra column, then a
//                        column-oriented back substitution.  O(N bw^2) work in
//                        place of the reference's dense O(N^3) solve;
//   angular regrid       interpolate_angular (:147-157): six-point Lagrange
//                        interpolation in theta on the pole-extended field, then
//                        in phi on the wrapped field, in the reference's order.
#include <algorithm>
#include <cmath>
#include <map>
#include <mutex>
#include <set>
#include <string>
#include <tuple>

#include <cuda_runtime.h>

#include "../../include/bssn_gb300.h"
#include "bssn_driver.h"
#include "bssn_profile.h"

namespace bssn {
namespace {

constexpr int kHThreads = 128;
constexpr int kSurfWarps = 4;     // nodes (one warp each) per block of the surface kernel
constexpr int kSumThreads = 1024;
constexpr int kStepWarps = 2;      // columns per block of a factorisation step (spread over the SMs)
constexpr int kBackThreads = 1024;
constexpr double kPi = 3.141592653589793;

struct HGeom {
    const double* g;  // (3, 3, *grid)
    const double* k;
    int dims;
    int n[3];
    double origin[3], spacing[3];
    int margin;
    long long cs;  // component stride
};

__device__ __forceinline__ double rmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double radd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double rdiv(double a, double b) { return __ddiv_rn(a, b); }

// Programmatic dependent launch: a step kernel waits for its predecessor's
// completion (and the visibility of its writes) before touching the band, and
// lets the next one be scheduled once its own stores are issued.  Without the
// launch attribute both instructions are no-ops.
__device__ __forceinline__ void pdl_enter() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_release() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

// ---------------------------------------------------------------------------
// Hermite weights and their index derivatives (hermite_interpolation.py:12-24)
// ---------------------------------------------------------------------------
__device__ inline int hermite(double index, int size, double (&w)[6], double (&dw)[6]) {
    const double fl = floor(index);
    int cell;
    if (!(fl >= 2.0)) cell = 2;
    else if (fl > (double)(size - 4)) cell = size - 4;
    else cell = (int)fl;
    const double t = index - (double)cell, t2 = t * t, t3 = t2 * t;
    const double h00 = 2 * t3 - 3 * t2 + 1, h01 = -2 * t3 + 3 * t2;
    const double h10 = t3 - 2 * t2 + t, h11 = t3 - t2;
    const double d00 = 6 * t2 - 6 * t, d01 = -6 * t2 + 6 * t;
    const double d10 = 3 * t2 - 4 * t + 1, d11 = 3 * t2 - 2 * t;
    const double L[6] = {1.0 / 12, -8.0 / 12, 0.0, 8.0 / 12, -1.0 / 12, 0.0};
    const double R[6] = {0.0, 1.0 / 12, -8.0 / 12, 0.0, 8.0 / 12, -1.0 / 12};
#pragma unroll
    for (int a = 0; a < 6; ++a) {
        w[a] = h10 * L[a] + h11 * R[a];
        dw[a] = d10 * L[a] + d11 * R[a];
    }
    w[2] += h00;
    w[3] += h01;
    dw[2] += d00;
    dw[3] += d01;
    return cell - 2;
}

__device__ __constant__ int kSym[6] = {0, 1, 2, 4, 5, 8};  // (00, 01, 02, 11, 12, 22)

__device__ inline void unpack(const double (&v)[6], double (&M)[3][3]) {
    M[0][0] = v[0]; M[0][1] = M[1][0] = v[1]; M[0][2] = M[2][0] = v[2];
    M[1][1] = v[3]; M[1][2] = M[2][1] = v[4]; M[2][2] = v[5];
}

__device__ __forceinline__ void warp_sum(double& v) {
    // butterfly: every lane ends with the same, order-independent sum of pairs
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
}

// gamma, d_gamma[k][i][j] = d_k gamma_ij, K and the resolved flag at a point
// (apparent_horizon.py:65-98).  The upper triangle of each tensor is read.
// S = 1: one thread samples the point; S = 32: the lanes of a warp split the
// Hermite stencil and every lane ends with the whole result.
template <int S>
__device__ void sample_point(const HGeom& G, const double (&p)[3], double (&gam)[3][3], double (&dg)[3][3][3],
                             double (&K)[3][3], bool& inside) {
    const int l0 = S == 1 ? 0 : (int)(threadIdx.x & 31);
    double idx[3], coord0 = 0.0;
    if (G.dims == 1) {
        coord0 = sqrt(p[0] * p[0] + p[1] * p[1] + p[2] * p[2]);
        idx[0] = (coord0 - G.origin[0]) / G.spacing[0];
        double w[6], dw[6];
        const int b = hermite(idx[0], G.n[0], w, dw);
        double v[4] = {0, 0, 0, 0}, d[2] = {0, 0};
        for (int a = l0; a < 6; a += S) {
            const long long o = b + a;
            const double grr = G.g[o], gtt = G.g[4 * G.cs + o];
            v[0] += w[a] * grr; v[1] += w[a] * gtt;
            d[0] += dw[a] * grr; d[1] += dw[a] * gtt;
            v[2] += w[a] * G.k[o]; v[3] += w[a] * G.k[4 * G.cs + o];
        }
        if (S > 1) {
            for (int q = 0; q < 4; ++q) warp_sum(v[q]);
            warp_sum(d[0]);
            warp_sum(d[1]);
        }
        d[0] /= G.spacing[0];
        d[1] /= G.spacing[0];
        const double r = fmax(coord0, 1e-30);
        const double nr[3] = {p[0] / r, p[1] / r, p[2] / r};
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) {
                const double rr = nr[i] * nr[j], e = i == j ? 1.0 : 0.0;
                gam[i][j] = v[0] * rr + v[1] * (e - rr);
                K[i][j] = v[2] * rr + v[3] * (e - rr);
            }
        // d_k gamma_ij = (g_rr' - g_tt') n_k n_i n_j + g_tt' n_k delta_ij
        //              + (g_rr - g_tt) d_k (n_i n_j),  d_k n_i = (delta_ik - n_i n_k) / r
        for (int k = 0; k < 3; ++k)
            for (int i = 0; i < 3; ++i)
                for (int j = 0; j < 3; ++j) {
                    const double dni = ((i == k ? 1.0 : 0.0) - nr[i] * nr[k]) / r;
                    const double dnj = ((j == k ? 1.0 : 0.0) - nr[j] * nr[k]) / r;
                    dg[k][i][j] = (d[0] - d[1]) * nr[k] * nr[i] * nr[j] + (i == j ? d[1] * nr[k] : 0.0) +
                                  (v[0] - v[1]) * (dni * nr[j] + nr[i] * dnj);
                }
    } else if (G.dims == 2) {
        coord0 = sqrt(p[0] * p[0] + p[1] * p[1]);
        idx[0] = (coord0 - G.origin[0]) / G.spacing[0];
        idx[1] = (p[2] - G.origin[1]) / G.spacing[1];
        double w0[6], d0[6], w1[6], d1[6];
        const int b0 = hermite(idx[0], G.n[0], w0, d0);
        const int b1 = hermite(idx[1], G.n[1], w1, d1);
        double gv[6] = {0}, gr[6] = {0}, gz[6] = {0}, kv[6] = {0};
        for (int t = l0; t < 36; t += S) {
            const int a = t / 6, c = t % 6;
            {
                const long long o = (long long)(b0 + a) * G.n[1] + (b1 + c);
                const double ww = w0[a] * w1[c], wr = d0[a] * w1[c], wz = w0[a] * d1[c];
#pragma unroll
                for (int q = 0; q < 6; ++q) {
                    const double gq = G.g[kSym[q] * G.cs + o];
                    gv[q] += ww * gq; gr[q] += wr * gq; gz[q] += wz * gq;
                    kv[q] += ww * G.k[kSym[q] * G.cs + o];
                }
            }
        }
        if (S > 1)
            for (int q = 0; q < 6; ++q) { warp_sum(gv[q]); warp_sum(gr[q]); warp_sum(gz[q]); warp_sum(kv[q]); }
#pragma unroll
        for (int q = 0; q < 6; ++q) { gr[q] /= G.spacing[0]; gz[q] /= G.spacing[1]; }
        double M[3][3], Mr[3][3], Mz[3][3], Kp[3][3];
        unpack(gv, M); unpack(gr, Mr); unpack(gz, Mz); unpack(kv, Kp);
        const double rho = fmax(coord0, 1e-30), c = p[0] / rho, s = p[1] / rho;
        const double Rm[3][3] = {{c, -s, 0.0}, {s, c, 0.0}, {0.0, 0.0, 1.0}};
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) {
                double a = 0.0, b = 0.0;
                for (int m = 0; m < 3; ++m)
                    for (int n = 0; n < 3; ++n) { a += Rm[i][m] * M[m][n] * Rm[j][n]; b += Rm[i][m] * Kp[m][n] * Rm[j][n]; }
                gam[i][j] = a;
                K[i][j] = b;
            }
        // d_k (R M R^T) with dc/dx = s^2/rho, dc/dy = -cs/rho, ds/dx = -cs/rho,
        // ds/dy = c^2/rho, drho = (c, s, 0), M depending on (rho, z).
        const double dc[3] = {s * s / rho, -c * s / rho, 0.0}, ds[3] = {-c * s / rho, c * c / rho, 0.0};
        const double drho[3] = {c, s, 0.0};
        for (int k = 0; k < 3; ++k) {
            const double dR[3][3] = {{dc[k], -ds[k], 0.0}, {ds[k], dc[k], 0.0}, {0.0, 0.0, 0.0}};
            for (int i = 0; i < 3; ++i)
                for (int j = 0; j < 3; ++j) {
                    double acc = 0.0;
                    for (int m = 0; m < 3; ++m)
                        for (int n = 0; n < 3; ++n) {
                            const double dM = Mr[m][n] * drho[k] + (k == 2 ? Mz[m][n] : 0.0);
                            acc += dR[i][m] * M[m][n] * Rm[j][n] + Rm[i][m] * dM * Rm[j][n] + Rm[i][m] * M[m][n] * dR[j][n];
                        }
                    dg[k][i][j] = acc;
                }
        }
    } else {
        for (int a = 0; a < 3; ++a) idx[a] = (p[a] - G.origin[a]) / G.spacing[a];
        double w0[6], d0[6], w1[6], d1[6], w2[6], d2[6];
        const int b0 = hermite(idx[0], G.n[0], w0, d0);
        const int b1 = hermite(idx[1], G.n[1], w1, d1);
        const int b2 = hermite(idx[2], G.n[2], w2, d2);
        double gv[6] = {0}, gx[6] = {0}, gy[6] = {0}, gz[6] = {0}, kv[6] = {0};
        for (int t = l0; t < 216; t += S) {
            const int a = t / 36, b = (t / 6) % 6, c = t % 6;
            {
                const long long row = ((long long)(b0 + a) * G.n[1] + (b1 + b)) * G.n[2] + b2;
                const double wab = w0[a] * w1[b], xab = d0[a] * w1[b], yab = w0[a] * d1[b];
                {
                    const long long o = row + c;
                    const double ww = wab * w2[c], wx = xab * w2[c], wy = yab * w2[c], wz = wab * d2[c];
#pragma unroll
                    for (int q = 0; q < 6; ++q) {
                        const double gq = G.g[kSym[q] * G.cs + o];
                        gv[q] += ww * gq; gx[q] += wx * gq; gy[q] += wy * gq; gz[q] += wz * gq;
                        kv[q] += ww * G.k[kSym[q] * G.cs + o];
                    }
                }
            }
        }
        if (S > 1)
            for (int q = 0; q < 6; ++q) {
                warp_sum(gv[q]); warp_sum(gx[q]); warp_sum(gy[q]); warp_sum(gz[q]); warp_sum(kv[q]);
            }
        double Dx[6], Dy[6], Dz[6];
#pragma unroll
        for (int q = 0; q < 6; ++q) { Dx[q] = gx[q] / G.spacing[0]; Dy[q] = gy[q] / G.spacing[1]; Dz[q] = gz[q] / G.spacing[2]; }
        unpack(gv, gam); unpack(kv, K);
        unpack(Dx, dg[0]); unpack(Dy, dg[1]); unpack(Dz, dg[2]);
    }
    inside = true;
    for (int a = 0; a < G.dims; ++a)
        inside = inside && idx[a] >= (double)G.margin && idx[a] <= (double)(G.n[a] - 1 - G.margin);
    if (G.dims < 3) inside = inside && coord0 > 1e-10 * G.spacing[0];
}

// ---------------------------------------------------------------------------
// angular grid and derivatives (apparent_horizon.py:101-144)
// ---------------------------------------------------------------------------
struct Sphere {
    int nt, np;
    const double* radius;
    const double* dir;  // optional: evaluate radius + step * dir
    double step;
};

__device__ __forceinline__ double hval(const Sphere& S, int t, int p) {
    const long long i = (long long)t * S.np + p;
    return S.dir ? radd(S.radius[i], rmul(S.step, S.dir[i])) : S.radius[i];
}

// Node of polar index r (which may be a ghost) and azimuth p.
__device__ __forceinline__ void fold(const Sphere& S, int r, int p, int& rt, int& rp) {
    if (r < 0) { rt = -1 - r; rp = (p + S.np / 2) % S.np; }
    else if (r >= S.nt) { rt = 2 * S.nt - 1 - r; rp = (p + S.np / 2) % S.np; }
    else { rt = r; rp = p; }
}

__device__ __constant__ double kFirst[5] = {1.0 / 12, -2.0 / 3, 0.0, 2.0 / 3, -1.0 / 12};
__device__ __constant__ double kSecond[5] = {-1.0 / 12, 4.0 / 3, -2.5, 4.0 / 3, -1.0 / 12};

__device__ double h_phi_at(const Sphere& S, int t, int p, double dph) {
    double acc = 0.0;
    for (int k = 0; k < 5; ++k) {
        if (k == 2) continue;
        acc = radd(acc, rmul(kFirst[k], hval(S, t, (p + k - 2 + S.np) % S.np)));
    }
    return rdiv(acc, dph);
}

// h_t, h_tt, h_p, h_pp, h_tp at node (t, p), summed as the reference sums them.
__device__ void ang_derivs(const Sphere& S, int t, int p, double (&D)[5]) {
    const double dth = rdiv(kPi, (double)S.nt), dph = rdiv(2.0 * kPi, (double)S.np);
    double a0 = 0.0, a1 = 0.0, a2 = 0.0, a3 = 0.0, a4 = 0.0;
    for (int k = 0; k < 5; ++k) {
        int rt, rp;
        fold(S, t + k - 2, p, rt, rp);
        const double v = hval(S, rt, rp);
        if (k != 2) {
            a0 = radd(a0, rmul(kFirst[k], v));
            a4 = radd(a4, rmul(kFirst[k], h_phi_at(S, rt, rp, dph)));
            a2 = radd(a2, rmul(kFirst[k], hval(S, t, (p + k - 2 + S.np) % S.np)));
        }
        a1 = radd(a1, rmul(kSecond[k], v));
        a3 = radd(a3, rmul(kSecond[k], hval(S, t, (p + k - 2 + S.np) % S.np)));
    }
    D[0] = rdiv(a0, dth);
    D[1] = rdiv(a1, rmul(dth, dth));
    D[2] = rdiv(a2, dph);
    D[3] = rdiv(a3, rmul(dph, dph));
    D[4] = rdiv(a4, dth);
}

struct Frame {
    double radial[3], polar[3], azim[3], sine, cot;
};

__device__ inline Frame frame(int t, int p, int nt, int np) {
    const double th = rdiv(rmul((double)t + 0.5, kPi), (double)nt);
    const double ph = rdiv(rmul((double)(2 * p), kPi), (double)np);
    double st, ct, sp, cp;
    sincos(th, &st, &ct);
    sincos(ph, &sp, &cp);
    Frame F;
    F.radial[0] = st * cp; F.radial[1] = st * sp; F.radial[2] = ct;
    F.polar[0] = ct * cp; F.polar[1] = ct * sp; F.polar[2] = -st;
    F.azim[0] = -sp; F.azim[1] = cp; F.azim[2] = 0.0;
    F.sine = st;
    F.cot = ct / st;
    return F;
}

// Positive definite (leading principal minors), the reference's Cholesky test.
__device__ inline bool positive(const double (&g)[3][3]) {
    const double m2 = g[0][0] * g[1][1] - g[0][1] * g[1][0];
    const double det = g[0][0] * (g[1][1] * g[2][2] - g[1][2] * g[2][1]) -
                       g[0][1] * (g[1][0] * g[2][2] - g[1][2] * g[2][0]) +
                       g[0][2] * (g[1][0] * g[2][1] - g[1][1] * g[2][0]);
    return g[0][0] > 0.0 && m2 > 0.0 && det > 0.0;
}

// Expansion and area density at one node (apparent_horizon.py:185-232).
__device__ void pointwise(double h, const double (&D)[5], const Frame& F, const double (&gam)[3][3],
                          const double (&dg)[3][3][3], const double (&K)[3][3], double& theta, double* density) {
    const double ht = D[0], htt = D[1], hp = D[2], hpp = D[3], htp = D[4];
    const double h2 = h * h, sn = F.sine;
    double grad[3];
    for (int a = 0; a < 3; ++a) grad[a] = F.radial[a] - (ht / h) * F.polar[a] - (hp / (h * sn)) * F.azim[a];
    const double crp = ht / h2, cra = hp / (h2 * sn), cpp = (1.0 / h - htt / h2) * 0.5;
    const double cpa = (F.cot * hp - htp) / (h2 * sn), caa = (1.0 / h - F.cot * ht / h2 - hpp / (h2 * sn * sn)) * 0.5;
    double inv[3][3];
    {
        const double c00 = gam[1][1] * gam[2][2] - gam[1][2] * gam[2][1];
        const double c01 = gam[1][2] * gam[2][0] - gam[1][0] * gam[2][2];
        const double c02 = gam[1][0] * gam[2][1] - gam[1][1] * gam[2][0];
        const double det = gam[0][0] * c00 + gam[0][1] * c01 + gam[0][2] * c02;
        const double id = 1.0 / det;
        inv[0][0] = c00 * id; inv[1][0] = c01 * id; inv[2][0] = c02 * id;
        inv[0][1] = (gam[0][2] * gam[2][1] - gam[0][1] * gam[2][2]) * id;
        inv[1][1] = (gam[0][0] * gam[2][2] - gam[0][2] * gam[2][0]) * id;
        inv[2][1] = (gam[0][1] * gam[2][0] - gam[0][0] * gam[2][1]) * id;
        inv[0][2] = (gam[0][1] * gam[1][2] - gam[0][2] * gam[1][1]) * id;
        inv[1][2] = (gam[0][2] * gam[1][0] - gam[0][0] * gam[1][2]) * id;
        inv[2][2] = (gam[0][0] * gam[1][1] - gam[0][1] * gam[1][0]) * id;
    }
    double up[3];
    for (int i = 0; i < 3; ++i) up[i] = inv[i][0] * grad[0] + inv[i][1] * grad[1] + inv[i][2] * grad[2];
    const double norm = sqrt(grad[0] * up[0] + grad[1] * up[1] + grad[2] * up[2]);
    double nu[3];
    for (int i = 0; i < 3; ++i) nu[i] = up[i] / norm;
    double div = 0.0, knn = 0.0, trk = 0.0;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            const double r = F.radial[i], q = F.polar[i], a = F.azim[i];
            const double rj = F.radial[j], qj = F.polar[j], aj = F.azim[j];
            const double hess = crp * (r * qj + q * rj) + cra * (r * aj + a * rj) + cpp * (q * qj + q * qj) +
                                cpa * (q * aj + a * qj) + caa * (a * aj + a * aj);
            double cg = 0.0;
            for (int l = 0; l < 3; ++l) cg += up[l] * (dg[i][l][j] + dg[j][l][i] - dg[l][i][j]);
            div += (inv[i][j] - nu[i] * nu[j]) * (hess - 0.5 * cg);
            knn += K[i][j] * nu[i] * nu[j];
            trk += inv[i][j] * K[i][j];
        }
    theta = div / norm + knn - trk;
    if (density) {
        double tt[3], tp[3];
        for (int a = 0; a < 3; ++a) {
            tt[a] = ht * F.radial[a] + h * F.polar[a];
            tp[a] = (hp / sn) * F.radial[a] + h * F.azim[a];
        }
        double mtt = 0.0, mpp = 0.0, mtp = 0.0;
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) {
                mtt += tt[i] * gam[i][j] * tt[j];
                mpp += tp[i] * gam[i][j] * tp[j];
                mtp += tt[i] * gam[i][j] * tp[j];
            }
        *density = sqrt(mtt * mpp - mtp * mtp);
    }
}

struct Band {
    double* a;      // column-major band, column j at a + j * ld, row i at offset i - j + ku2
    int n, kl, ku2, ld;
};

__device__ __forceinline__ double& band_at(const Band& B, int i, int j) {
    return B.a[(long long)j * B.ld + (i - j + B.ku2)];
}

// One warp per node: the surface, the node's bad flag, and (band != null) the
// node's Jacobian row.  The lanes share each geometry sample; for the row,
// lanes 1-10 evaluate the expansion with one angular derivative moved by -+ its
// step (lane 0 the unmoved one) in a single pass, then two more samples give
// the radial partial.
__global__ void __launch_bounds__(kSurfWarps * 32)
k_surface(HGeom G, Sphere S, double cx, double cy, double cz, double* __restrict__ trial,
          double* __restrict__ expansion, double* __restrict__ density, int* __restrict__ bad, Band B,
          double fd_step) {
    const int lane = threadIdx.x & 31;
    const int i = blockIdx.x * kSurfWarps + (threadIdx.x >> 5);
    if (i >= S.nt * S.np) return;  // whole warp
    const int t = i / S.np, p = i % S.np;
    const double h = hval(S, t, p);
    double D[5];
    ang_derivs(S, t, p, D);
    const Frame F = frame(t, p, S.nt, S.np);
    double gam[3][3], dg[3][3][3], K[3][3];
    bool inside;
    double pt[3] = {cx + h * F.radial[0], cy + h * F.radial[1], cz + h * F.radial[2]};
    sample_point<32>(G, pt, gam, dg, K, inside);
    // lane 1 + 2m: D[m] + step, lane 2 + 2m: D[m] - step (m = 0..4)
    double Dl[5] = {D[0], D[1], D[2], D[3], D[4]};
    const int m = (lane - 1) >> 1;
    if (B.a && lane >= 1 && lane <= 10) {
        const double sc = fd_step * fmax(fabs(D[m]), 1.0);
        Dl[m] = (lane & 1) ? D[m] + sc : D[m] - sc;
    }
    double th, dens;
    pointwise(h, Dl, F, gam, dg, K, th, &dens);
    const double th0 = __shfl_sync(0xffffffffu, th, 0);
    const double dens0 = __shfl_sync(0xffffffffu, dens, 0);
    double tpm[10];
#pragma unroll
    for (int q = 0; q < 10; ++q) tpm[q] = __shfl_sync(0xffffffffu, th, q + 1);
    if (lane == 0) {
        if (trial) trial[i] = h;
        expansion[i] = th0;
        if (density) density[i] = dens0;
        const bool ok = inside && positive(gam) && isfinite(th0) && isfinite(dens0) && h > 0.0;
        bad[i] = ok ? 0 : 1;
    }
    if (!B.a) return;

    double part[6];
    {
        const double dh = fd_step * fmax(fabs(h), 1.0);
        double gp[3][3], dgp[3][3][3], Kp[3][3], tp, tm;
        bool in2;
        const double hp_ = h + dh, hm_ = h - dh;
        double q[3] = {cx + hp_ * F.radial[0], cy + hp_ * F.radial[1], cz + hp_ * F.radial[2]};
        sample_point<32>(G, q, gp, dgp, Kp, in2);
        pointwise(hp_, D, F, gp, dgp, Kp, tp, nullptr);
        q[0] = cx + hm_ * F.radial[0]; q[1] = cy + hm_ * F.radial[1]; q[2] = cz + hm_ * F.radial[2];
        sample_point<32>(G, q, gp, dgp, Kp, in2);
        pointwise(hm_, D, F, gp, dgp, Kp, tm, nullptr);
        part[0] = (tp - tm) / (2.0 * dh);
    }
#pragma unroll
    for (int mm = 0; mm < 5; ++mm) {
        const double sc = fd_step * fmax(fabs(D[mm]), 1.0);
        part[mm + 1] = (tpm[2 * mm] - tpm[2 * mm + 1]) / (2.0 * sc);
    }
    if (lane != 0) return;

    // row i of the Jacobian: diagonal plus the partials times the stencils
    const double dth = rdiv(kPi, (double)S.nt), dph = rdiv(2.0 * kPi, (double)S.np);
    const double dth2 = rmul(dth, dth), dph2 = rmul(dph, dph);
    band_at(B, i, i) += part[0];
    for (int k = 0; k < 5; ++k) {
        int rt, rp;
        fold(S, t + k - 2, p, rt, rp);
        const int jt = rt * S.np + rp;
        if (k != 2) band_at(B, i, jt) += part[1] * (kFirst[k] / dth);
        band_at(B, i, jt) += part[2] * (kSecond[k] / dth2);
        const int ja = t * S.np + (p + k - 2 + S.np) % S.np;
        if (k != 2) band_at(B, i, ja) += part[3] * (kFirst[k] / dph);
        band_at(B, i, ja) += part[4] * (kSecond[k] / dph2);
        if (k == 2) continue;
        for (int b = 0; b < 5; ++b) {
            if (b == 2) continue;
            const int jm = rt * S.np + (rp + b - 2 + S.np) % S.np;
            band_at(B, i, jm) += part[5] * (kFirst[k] * (kFirst[b] / dph) / dth);
        }
    }
}

// Sum of radii, max |expansion|, bad node count and the area quadrature, in
// a fixed order (one block).
__global__ void __launch_bounds__(kSumThreads)
k_surface_summary(const double* __restrict__ radius, const double* __restrict__ expansion,
                  const double* __restrict__ density, const int* __restrict__ bad,
                  const double* __restrict__ weights, int nt, int np, double* __restrict__ out) {
    __shared__ double s_sum[kSumThreads], s_max[kSumThreads], s_bad[kSumThreads], s_area[kSumThreads];
    const int n = nt * np;
    double sum = 0.0, mx = 0.0, nb = 0.0, area = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        sum += radius[i];
        const double a = fabs(expansion[i]);
        mx = (a > mx || a != a) ? a : mx;
        nb += bad[i];
        if (density && weights) area += weights[i / np] * density[i];
    }
    s_sum[threadIdx.x] = sum; s_max[threadIdx.x] = mx; s_bad[threadIdx.x] = nb; s_area[threadIdx.x] = area;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) {
            s_sum[threadIdx.x] += s_sum[threadIdx.x + w];
            const double a = s_max[threadIdx.x + w];
            if (a > s_max[threadIdx.x] || a != a) s_max[threadIdx.x] = a;
            s_bad[threadIdx.x] += s_bad[threadIdx.x + w];
            s_area[threadIdx.x] += s_area[threadIdx.x + w];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        out[0] = s_sum[0];
        out[1] = s_max[0];
        out[2] = s_bad[0];
        out[3] = s_area[0] * rdiv(2.0 * kPi, (double)np);
    }
}

// ---------------------------------------------------------------------------
// band LU with partial pivoting, one launch per column k: every warp finds the
// pivot of column k itself (first largest modulus), then applies the row swap
// and the elimination to its own column j in (k, k + ku2], or (the last warp)
// to the right-hand side.  Column k is only read during step k; its pivot goes
// to diag[k].
// ---------------------------------------------------------------------------
constexpr int kRowsPerLane = 12;  // rows per lane per pass: loads issued together

__global__ void __launch_bounds__(kStepWarps * 32)
k_band_step(Band B, int k, double* __restrict__ rhs, double* __restrict__ diag) {
    pdl_enter();
    const int lane = threadIdx.x & 31;
    const int col = k + 1 + blockIdx.x * kStepWarps + (threadIdx.x >> 5);
    const int last = min(B.n - 1, k + B.ku2);
    const bool is_rhs = col == last + 1;
    if (col > last + 1) return;
    const int rmax = min(B.n - 1, k + B.kl);
    const double* __restrict__ ck = B.a + (long long)k * B.ld + B.ku2 - k;  // ck[r] = A(r, k)
    double best = -1.0;
    int arg = k;
    for (int base = k; base <= rmax; base += 32 * kRowsPerLane) {
        double v[kRowsPerLane];
#pragma unroll
        for (int q = 0; q < kRowsPerLane; ++q) {
            const int r = base + lane + 32 * q;
            v[q] = r <= rmax ? fabs(ck[r]) : -1.0;
        }
#pragma unroll
        for (int q = 0; q < kRowsPerLane; ++q)
            if (v[q] > best) { best = v[q]; arg = base + lane + 32 * q; }
    }
    for (int o = 16; o > 0; o >>= 1) {
        const double ob = __shfl_xor_sync(0xffffffffu, best, o);
        const int oa = __shfl_xor_sync(0xffffffffu, arg, o);
        if (ob > best || (ob == best && oa < arg)) { best = ob; arg = oa; }
    }
    const int pr = arg;
    double* __restrict__ cj = is_rhs ? rhs : B.a + (long long)col * B.ld + (B.ku2 - col);  // cj[r] = A(r, col)
    const double piv = ck[pr], akk = ck[k], xk = cj[k], xp = cj[pr];
    const double rpiv = 1.0 / piv;  // multipliers scaled by the reciprocal, as getf2 does
    __syncwarp();  // every lane holds rows k and pr before any lane rewrites them
    for (int base = k + 1; base <= rmax; base += 32 * kRowsPerLane) {
        double a[kRowsPerLane], x[kRowsPerLane];
#pragma unroll
        for (int q = 0; q < kRowsPerLane; ++q) {
            const int r = base + lane + 32 * q;
            a[q] = r <= rmax ? ck[r] : 0.0;
            x[q] = r <= rmax ? cj[r] : 0.0;
        }
#pragma unroll
        for (int q = 0; q < kRowsPerLane; ++q) {
            const int r = base + lane + 32 * q;
            if (r <= rmax) {
                const double l = (r == pr ? akk : a[q]) * rpiv;
                cj[r] = (r == pr ? xk : x[q]) - l * xp;
            }
        }
    }
    __syncwarp();
    if (lane == 0) {
        cj[k] = xp;
        if (is_rhs) diag[k] = piv;
    }
}

// The same step with the pivot search of the next column folded in: the warp
// that updates column k + 1 holds its new entries in registers, finds their
// first largest modulus and leaves the row in piv_row[k + 1], so every step
// makes one round trip to memory (the pivot row's entries come from the lane
// that loaded them).  Step 0 searches its own column (search = 1).  Needs
// kl + 2 <= 32 * kRowsPerLane.
__global__ void __launch_bounds__(kStepWarps * 32)
k_band_step_fused(Band B, int k, int search, double* __restrict__ rhs, double* __restrict__ diag,
                  int* __restrict__ piv_row) {
    pdl_enter();
    const int lane = threadIdx.x & 31;
    const int col = k + 1 + blockIdx.x * kStepWarps + (threadIdx.x >> 5);
    const int last = min(B.n - 1, k + B.ku2);
    const bool is_rhs = col == last + 1;
    if (col > last + 1) return;
    const bool next = !is_rhs && col == k + 1;  // this warp searches the next pivot
    const int rmax = min(B.n - 1, k + B.kl);
    const int rext = next ? min(B.n - 1, col + B.kl) : rmax;  // rows of column k + 1 to search
    const double* __restrict__ ck = B.a + (long long)k * B.ld + B.ku2 - k;  // ck[r] = A(r, k)
    double* __restrict__ cj = is_rhs ? rhs : B.a + (long long)col * B.ld + (B.ku2 - col);
    const int pre = search ? -1 : piv_row[k];
    double a[kRowsPerLane], x[kRowsPerLane];
#pragma unroll
    for (int q = 0; q < kRowsPerLane; ++q) {
        const int r = k + lane + 32 * q;
        a[q] = r <= rmax ? ck[r] : 0.0;
        x[q] = r <= rext ? cj[r] : 0.0;
    }
    int pr = pre;
    if (search) {
        double best = -1.0;
        int arg = k;
#pragma unroll
        for (int q = 0; q < kRowsPerLane; ++q) {
            const int r = k + lane + 32 * q;
            const double v = r <= rmax ? fabs(a[q]) : -1.0;
            if (v > best) { best = v; arg = r; }
        }
        for (int o = 16; o > 0; o >>= 1) {
            const double ob = __shfl_xor_sync(0xffffffffu, best, o);
            const int oa = __shfl_xor_sync(0xffffffffu, arg, o);
            if (ob > best || (ob == best && oa < arg)) { best = ob; arg = oa; }
        }
        pr = arg;
    }
    // rows k and pr of both columns from the lanes that hold them
    const int qp = (pr - k) >> 5, lp = (pr - k) & 31;
    double ap = 0.0, xpv = 0.0;
#pragma unroll
    for (int q = 0; q < kRowsPerLane; ++q)
        if (q == qp) { ap = a[q]; xpv = x[q]; }
    const double piv = __shfl_sync(0xffffffffu, ap, lp);
    const double xp = __shfl_sync(0xffffffffu, xpv, lp);
    const double akk = __shfl_sync(0xffffffffu, a[0], 0);
    const double xk = __shfl_sync(0xffffffffu, x[0], 0);
    const double rpiv = 1.0 / piv;  // multipliers scaled by the reciprocal, as getf2 does
    double best = -1.0;
    int arg = col;
#pragma unroll
    for (int q = 0; q < kRowsPerLane; ++q) {
        const int r = k + lane + 32 * q;
        if (r > k && r <= rmax) {
            const double l = (r == pr ? akk : a[q]) * rpiv;
            x[q] = (r == pr ? xk : x[q]) - l * xp;
            cj[r] = x[q];
        }
        if (next && r > k && r <= rext) {
            const double v = fabs(x[q]);
            if (v > best) { best = v; arg = r; }
        }
    }
    if (lane == 0) {
        cj[k] = xp;
        if (is_rhs) diag[k] = piv;
    }
    if (next) {
        for (int o = 16; o > 0; o >>= 1) {
            const double ob = __shfl_xor_sync(0xffffffffu, best, o);
            const int oa = __shfl_xor_sync(0xffffffffu, arg, o);
            if (ob > best || (ob == best && oa < arg)) { best = ob; arg = oa; }
        }
        if (lane == 0) piv_row[col] = arg;
    }
    pdl_release();
}

// Blocked form: one launch factors kPanel columns.  Every block factors the
// panel (rows c0 .. c0 + kl + kPanel - 1 of columns c0 .. c0 + kPanel - 1)
// from a copy the previous launch left in `pin` (the same pivot rule, swaps
// and eliminations as the column steps, in the same order), then each warp
// applies the panel's swaps and eliminations to one trailing column (or the
// right-hand side).  The warps whose columns form the next panel also write
// them to `pout`; block 0 writes the panel's U rows and pivots back.  Needs
// kl + kPanel <= kPanelRows.
//
// The panel lives in registers: thread t holds rows t, t + 128, t + 256 of all
// kPanel columns, so a column step is one barrier.  Each warp reduces a pivot
// candidate and its owner publishes the candidate row (and the owner of row jj
// that row) to double-buffered shared slots; after the barrier every thread
// picks the winner and eliminates its own rows.  A trailing column lives in
// registers too (lane l holds rows l + 32 q): the row swap and the pivot-row
// broadcast are shuffles, and only the L multipliers are read from shared memory.
constexpr int kPanel = 8;
constexpr int kPanelWarps = 4;
constexpr int kPanelRows = 384;

// v[q] for a q known only at run time, without dynamic register indexing.
template <int N>
__device__ __forceinline__ double pick(const double (&v)[N], int q) {
    double out = 0.0;
#pragma unroll
    for (int i = 0; i < N; ++i)
        if (i == q) out = v[i];
    return out;
}
template <int N>
__device__ __forceinline__ void place(double (&v)[N], int q, double x) {
#pragma unroll
    for (int i = 0; i < N; ++i)
        if (i == q) v[i] = x;
}

__global__ void __launch_bounds__(kPanelWarps * 32)
k_band_panel(Band B, int c0, const double* __restrict__ pin, double* __restrict__ pout, double* __restrict__ rhs,
             double* __restrict__ diag) {
    pdl_enter();
    constexpr int kThr = kPanelWarps * 32;
    constexpr int kQP = (kPanelRows + kThr - 1) / kThr;   // panel rows per thread
    constexpr int kQC = kPanelRows / 32;                  // trailing-column rows per lane
    __shared__ double Ps[kPanel][kPanelRows];              // factored panel: L below, U on and above the diagonal
    __shared__ double Cs[kPanelWarps][kPanelRows];
    __shared__ double s_cand[2][kPanelWarps][kPanel];      // each warp's pivot candidate row
    __shared__ double s_cbest[2][kPanelWarps];
    __shared__ int s_carg[2][kPanelWarps];
    __shared__ double s_rowk[2][kPanel];                   // row jj before the step
    __shared__ int s_po[kPanel];
    __shared__ double s_piv[kPanel];
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    const int P = B.kl + kPanel;
    const int nrow = min(P, B.n - c0);
    const int ncol = min(kPanel, B.n - c0);

    double v[kPanel][kQP];
#pragma unroll
    for (int jj = 0; jj < kPanel; ++jj)
#pragma unroll
        for (int q = 0; q < kQP; ++q) {
            const int o = tid + q * kThr;
            v[jj][q] = (jj < ncol && o < nrow) ? pin[jj * P + o] : 0.0;
        }
#pragma unroll
    for (int jj = 0; jj < kPanel; ++jj) {
        if (jj >= ncol) break;
        const int omax = min(nrow - 1, jj + B.kl);
        const int sb = jj & 1;
        // this thread's candidate, then the warp's (largest |value|, lowest row on ties)
        double best = -1.0;
        int arg = jj;
#pragma unroll
        for (int q = 0; q < kQP; ++q) {
            const int o = tid + q * kThr;
            if (o >= jj && o <= omax) {
                const double a = fabs(v[jj][q]);
                if (a > best) { best = a; arg = o; }
            }
        }
        for (int sh = 16; sh > 0; sh >>= 1) {
            const double ob = __shfl_xor_sync(0xffffffffu, best, sh);
            const int oa = __shfl_xor_sync(0xffffffffu, arg, sh);
            if (ob > best || (ob == best && oa < arg)) { best = ob; arg = oa; }
        }
        if (lane == 0) {
            s_cbest[sb][w] = best;
            s_carg[sb][w] = arg;
        }
        if (best >= 0.0 && tid == arg % kThr) {
#pragma unroll
            for (int jc = 0; jc < kPanel; ++jc) s_cand[sb][w][jc] = pick(v[jc], arg / kThr);
        }
        if (tid == jj % kThr) {
#pragma unroll
            for (int jc = 0; jc < kPanel; ++jc) s_rowk[sb][jc] = v[jc][jj / kThr];
        }
        __syncthreads();
        int win = 0;
        double wb = s_cbest[sb][0];
        int wa = s_carg[sb][0];
#pragma unroll
        for (int ww = 1; ww < kPanelWarps; ++ww) {
            const double ob = s_cbest[sb][ww];
            const int oa = s_carg[sb][ww];
            if (ob > wb || (ob == wb && oa < wa)) { wb = ob; wa = oa; win = ww; }
        }
        const int po = wa;
        double xp[kPanel], xk[kPanel];
#pragma unroll
        for (int jc = 0; jc < kPanel; ++jc) {
            xp[jc] = s_cand[sb][win][jc];
            xk[jc] = s_rowk[sb][jc];
        }
        const double piv = xp[jj], akk = xk[jj];
        const double rp = 1.0 / piv;   // multipliers scaled by the reciprocal, as getf2 does
        if (tid == 0) {
            s_po[jj] = po;
            s_piv[jj] = piv;
        }
#pragma unroll
        for (int q = 0; q < kQP; ++q) {
            const int o = tid + q * kThr;
            if (o > jj && o <= omax) {
                const double l = (o == po ? akk : v[jj][q]) * rp;
                v[jj][q] = l;
#pragma unroll
                for (int jc = jj + 1; jc < kPanel; ++jc)
                    if (jc < ncol) v[jc][q] = (o == po ? xk[jc] : v[jc][q]) - l * xp[jc];
            } else if (o == jj) {
                v[jj][q] = piv;
#pragma unroll
                for (int jc = jj + 1; jc < kPanel; ++jc)
                    if (jc < ncol) v[jc][q] = xp[jc];
            }
        }
    }
#pragma unroll
    for (int jj = 0; jj < kPanel; ++jj)
#pragma unroll
        for (int q = 0; q < kQP; ++q) {
            const int o = tid + q * kThr;
            if (o < kPanelRows) Ps[jj][o] = v[jj][q];
        }
    __syncthreads();

    // trailing columns (and the right-hand side)
    const int first = c0 + ncol;
    const int lastc = min(B.n - 1, c0 + ncol - 1 + B.ku2);
    const int ntrail = lastc >= first ? lastc - first + 1 : 0;
    const int idx = blockIdx.x * kPanelWarps + w;
    if (idx <= ntrail) {
        const bool is_rhs = idx == ntrail;
        const int j = first + idx;
        double* col = is_rhs ? rhs : B.a + (long long)j * B.ld + (B.ku2 - j);  // col[r] = A(r, j)
        const int rlo = is_rhs ? 0 : j - B.ku2;                                 // rows inside the band
        const int rhi = is_rhs ? B.n - 1 : min(B.n - 1, j + B.kl);
        double cr[kQC];
#pragma unroll
        for (int q = 0; q < kQC; ++q) {
            const int o = lane + 32 * q, r = c0 + o;
            cr[q] = (o < nrow && r >= rlo && r <= rhi) ? col[r] : 0.0;
        }
#pragma unroll
        for (int jj = 0; jj < kPanel; ++jj) {
            if (jj >= ncol) break;
            const int po = s_po[jj];
            // swap rows jj (lane jj, slot 0) and po, then eliminate below jj
            const double a_jj = __shfl_sync(0xffffffffu, cr[0], jj);
            const double a_po = __shfl_sync(0xffffffffu, pick(cr, po >> 5), po & 31);
            if (lane == jj) cr[0] = a_po;
            if (po != jj && lane == (po & 31)) place(cr, po >> 5, a_jj);
            const double xc = a_po;
            const int omax = min(nrow - 1, jj + B.kl);
#pragma unroll
            for (int q = 0; q < kQC; ++q) {
                const int o = lane + 32 * q;
                if (o > jj && o <= omax) cr[q] -= Ps[jj][o] * xc;
            }
        }
        double* cs = Cs[w];
#pragma unroll
        for (int q = 0; q < kQC; ++q) {
            const int o = lane + 32 * q, r = c0 + o;
            if (o < nrow) {
                cs[o] = cr[q];
                if (r >= rlo && r <= rhi) col[r] = cr[q];
            }
        }
        __syncwarp();
        // the next panel's copy
        const int nc0 = first;
        if (!is_rhs && j < nc0 + kPanel) {
            const int nrow2 = min(P, B.n - nc0);
            double* dst = pout + (long long)(j - nc0) * P;
            for (int o = lane; o < nrow2; o += 32) {
                const int r = nc0 + o;
                const int local = r - c0;
                double x = 0.0;
                if (r >= rlo && r <= rhi) x = local < nrow ? cs[local] : col[r];
                dst[o] = x;
            }
        }
    }
    if (blockIdx.x == 0) {
        // U rows c0 .. c of each panel column c, and its pivot
        if (tid < ncol)
            for (int o = 0; o <= tid; ++o) B.a[(long long)(c0 + tid) * B.ld + (o - tid + B.ku2)] = Ps[tid][o];
        if (tid < ncol) diag[c0 + tid] = s_piv[tid];
    }
    pdl_release();
}

// Copy of the first panel (columns 0 .. kPanel - 1, rows 0 .. kl + kPanel - 1).
__global__ void k_panel_init(Band B, double* __restrict__ pout) {
    const int P = B.kl + kPanel;
    const int nrow = min(P, B.n), ncol = min(kPanel, B.n);
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < kPanel * P; e += gridDim.x * blockDim.x) {
        const int jj = e / P, o = e % P;
        double v = 0.0;
        if (jj < ncol && o < nrow && o - jj <= B.kl) v = B.a[(long long)jj * B.ld + (o - jj + B.ku2)];
        pout[e] = v;
    }
}

// Back substitution with y and 1/U_kk in shared memory, eight columns per
// pair of barriers: warp 0 solves the block's 8 x 8 triangle in registers
// (lane l holds row kl0 + l), then thread t subtracts the block's unknowns
// from row kl0 - 1 - t.  Every row receives its column terms in the same
// (descending) order as one column at a time.  The next block's U entries
// are loaded while the current one is solved.
constexpr int kBackBlock = 8;
constexpr int kBackSmemMax = 200 * 1024;

__global__ void __launch_bounds__(kBackThreads)
k_band_back_shared(Band B, double* __restrict__ y, const double* __restrict__ diag, double* __restrict__ out) {
    pdl_enter();
    extern __shared__ double sm[];
    double* sy = sm;
    double* srd = sm + B.n;
    __shared__ double sx[kBackBlock];
    __shared__ double s_max[kBackThreads], s_bad[kBackThreads];
    const int t = threadIdx.x, lane = t & 31;
    for (int i = t; i < B.n; i += blockDim.x) {
        sy[i] = y[i];
        srd[i] = 1.0 / diag[i];
    }
    // U entries of the block ending at column kh: pd[cl] = U(kl0 + lane, kl0 + cl)
    // above the diagonal (warp 0), pu[j] = U(kl0 - 1 - t, kh - j)
    auto load = [&](int kh, double (&pd)[kBackBlock], double (&pu)[kBackBlock]) {
        const int kl0 = max(0, kh - kBackBlock + 1);
#pragma unroll
        for (int cl = 0; cl < kBackBlock; ++cl) {
            const int r = kl0 + lane, c = kl0 + cl;
            pd[cl] = (t < 32 && c > r && c <= kh) ? B.a[(long long)c * B.ld + (r - c + B.ku2)] : 0.0;
        }
#pragma unroll
        for (int j = 0; j < kBackBlock; ++j) {
            const int r = kl0 - 1 - t, c = kh - j;
            pu[j] = (t < B.ku2 && r >= 0 && c >= kl0 && c - r <= B.ku2) ? B.a[(long long)c * B.ld + (r - c + B.ku2)]
                                                                       : 0.0;
        }
    };
    double pd[kBackBlock], pu[kBackBlock], nd[kBackBlock], nu[kBackBlock];
    int kh = B.n - 1;
    load(kh, pd, pu);
    __syncthreads();
    while (kh >= 0) {
        const int kl0 = max(0, kh - kBackBlock + 1), nb = kh - kl0 + 1, khn = kl0 - 1;
        if (khn >= 0) load(khn, nd, nu);
        if (t < 32) {
            double yv = lane < nb ? sy[kl0 + lane] : 0.0;
#pragma unroll
            for (int cl = kBackBlock - 1; cl >= 0; --cl) {
                if (cl >= nb) continue;
                const double x = __shfl_sync(0xffffffffu, yv, cl) * srd[kl0 + cl];
                if (lane == cl) yv = x;
                else if (lane < cl) yv -= pd[cl] * x;
            }
            if (lane < nb) {
                sy[kl0 + lane] = yv;
                sx[lane] = yv;
            }
        }
        __syncthreads();
        const int r = kl0 - 1 - t;
        if (t < B.ku2 && r >= 0) {
            double v = sy[r];
#pragma unroll
            for (int j = 0; j < kBackBlock; ++j)
                if (j < nb) v -= pu[j] * sx[nb - 1 - j];
            sy[r] = v;
        }
        __syncthreads();
        kh = khn;
#pragma unroll
        for (int q = 0; q < kBackBlock; ++q) { pd[q] = nd[q]; pu[q] = nu[q]; }
    }
    double mx = 0.0, nbad = 0.0;
    for (int i = t; i < B.n; i += blockDim.x) {
        const double v = sy[i];
        y[i] = v;
        if (!isfinite(v)) nbad += 1.0;
        else mx = fmax(mx, fabs(v));
    }
    s_max[t] = mx;
    s_bad[t] = nbad;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if (t < w) {
            s_max[t] = fmax(s_max[t], s_max[t + w]);
            s_bad[t] += s_bad[t + w];
        }
        __syncthreads();
    }
    if (t == 0) { out[0] = s_max[0]; out[1] = s_bad[0]; }
}

// x = U^-1 y by columns: x_k = y_k / U_kk, then y_r -= U_rk x_k above it.
// One block; also writes max |x| and the nonfinite count.
__global__ void __launch_bounds__(kBackThreads)
k_band_back(Band B, double* __restrict__ y, const double* __restrict__ diag, double* __restrict__ out) {
    pdl_enter();
    __shared__ double s_x;
    __shared__ double s_max[kBackThreads], s_bad[kBackThreads];
    for (int k = B.n - 1; k >= 0; --k) {
        if (threadIdx.x == 0) {
            const double x = y[k] / diag[k];
            y[k] = x;
            s_x = x;
        }
        __syncthreads();
        const double x = s_x;
        const int r0 = max(0, k - B.ku2);
        for (int r = r0 + threadIdx.x; r < k; r += blockDim.x)
            y[r] -= B.a[(long long)k * B.ld + (r - k + B.ku2)] * x;
        __syncthreads();
    }
    double mx = 0.0, nb = 0.0;
    for (int i = threadIdx.x; i < B.n; i += blockDim.x) {
        const double v = y[i];
        if (!isfinite(v)) nb += 1.0;
        else mx = fmax(mx, fabs(v));
    }
    s_max[threadIdx.x] = mx;
    s_bad[threadIdx.x] = nb;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) {
            s_max[threadIdx.x] = fmax(s_max[threadIdx.x], s_max[threadIdx.x + w]);
            s_bad[threadIdx.x] += s_bad[threadIdx.x + w];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) { out[0] = s_max[0]; out[1] = s_bad[0]; }
}

__global__ void k_negate(const double* __restrict__ src, double* __restrict__ dst, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) dst[i] = -src[i];
}

__global__ void k_band_dense(Band B, double* __restrict__ dense) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)B.n * B.n) return;
    const int i = (int)(t / B.n), j = (int)(t % B.n);
    const int off = i - j;
    dense[t] = (off >= -B.ku2 && off <= B.kl) ? band_at(B, i, j) : 0.0;
}

// ---------------------------------------------------------------------------
// geometry at arbitrary points and angular derivatives on their own
// ---------------------------------------------------------------------------
__global__ void k_sample(HGeom G, const double* __restrict__ points, long long n, double* __restrict__ gamma,
                         double* __restrict__ d_gamma, double* __restrict__ curvature, int* __restrict__ valid) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    const double p[3] = {points[3 * t], points[3 * t + 1], points[3 * t + 2]};
    double gam[3][3], dg[3][3][3], K[3][3];
    bool inside;
    sample_point<1>(G, p, gam, dg, K, inside);
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            if (gamma) gamma[9 * t + 3 * i + j] = gam[i][j];
            if (curvature) curvature[9 * t + 3 * i + j] = K[i][j];
            if (d_gamma)
                for (int k = 0; k < 3; ++k) d_gamma[27 * t + 9 * k + 3 * i + j] = dg[k][i][j];
        }
    if (valid) valid[t] = inside ? 1 : 0;
}

__global__ void k_ang(Sphere S, double* __restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int n = S.nt * S.np;
    if (i >= n) return;
    double D[5];
    ang_derivs(S, i / S.np, i % S.np, D);
    for (int m = 0; m < 5; ++m) out[(long long)m * n + i] = D[m];
}

// ---------------------------------------------------------------------------
// interpolate_angular (:147-157)
// ---------------------------------------------------------------------------
__device__ inline int lagrange6(double q, int size, double (&w)[6]) {
    int start = (int)floor(q) - 2;
    if (start < 0) start = 0;
    if (start > size - 6) start = size - 6;
#pragma unroll
    for (int k = 0; k < 6; ++k) {
        double c = 1.0;
#pragma unroll
        for (int m = 0; m < 6; ++m) {
            if (m == k) continue;
            c = rmul(c, rdiv(radd(q, -(double)(start + m)), (double)(k - m)));
        }
        w[k] = c;
    }
    return start;
}

__global__ void k_regrid(const double* __restrict__ src, int nt, int np, const double* __restrict__ theta, int nt2,
                         const double* __restrict__ phi, int np2, double* __restrict__ dst) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nt2 * np2) return;
    const int a = i / np2, b = i % np2;
    const double qt = radd(radd(rdiv(rmul(theta[a], (double)nt), kPi), -0.5), 3.0);
    const double qp = radd(rdiv(rmul(phi[b], (double)np), 2.0 * kPi), 3.0);
    const bool ok = qt >= 0.0 && qt <= (double)(nt + 5) && qp >= 0.0 && qp <= (double)(np + 5);
    double wt[6], wp[6];
    const int st = lagrange6(ok ? qt : 0.0, nt + 6, wt);
    const int sp = lagrange6(ok ? qp : 0.0, np + 6, wp);
    double acc = 0.0;
    for (int c = 0; c < 6; ++c) {
        const int ce = sp + c;  // column of the wrapped field
        const int col = ce < 3 ? np - 3 + ce : (ce < np + 3 ? ce - 3 : ce - np - 3);
        double v = 0.0;
        for (int r = 0; r < 6; ++r) {
            const int e = st + r - 3;  // polar index, ghosts folded
            int rt, rp;
            if (e < 0) { rt = -1 - e; rp = (col + np / 2) % np; }
            else if (e >= nt) { rt = 2 * nt - 1 - e; rp = (col + np / 2) % np; }
            else { rt = e; rp = col; }
            const double term = rmul(src[(long long)rt * np + rp], wt[r]);
            v = r == 0 ? term : radd(v, term);
        }
        const double term = rmul(v, wp[c]);
        acc = c == 0 ? term : radd(acc, term);
    }
    dst[i] = ok ? acc : __longlong_as_double(0x7ff8000000000000LL);
}

// ---------------------------------------------------------------------------
// host helpers
// ---------------------------------------------------------------------------
int geometry_of(const BssnHorizonGeometry* g, HGeom& G, const char* where) {
    if (!g || !g->gamma || !g->curvature) return fail(BSSN_ERR_INVALID, std::string(where) + ": null geometry");
    if (g->dims < 1 || g->dims > 3) return fail(BSSN_ERR_INVALID, std::string(where) + ": dims must be 1, 2 or 3");
    G.g = g->gamma;
    G.k = g->curvature;
    G.dims = g->dims;
    G.margin = g->margin;
    long long cs = 1;
    for (int a = 0; a < 3; ++a) {
        const int n = a < g->dims ? g->size[a] : 1;
        if (a < g->dims && (n < 6 || !(g->spacing[a] > 0.0)))
            return fail(BSSN_ERR_INVALID, std::string(where) + ": each axis needs six points and a positive spacing");
        G.n[a] = n;
        G.origin[a] = a < g->dims ? g->origin[a] : 0.0;
        G.spacing[a] = a < g->dims ? g->spacing[a] : 1.0;
        cs *= n;
    }
    if (g->margin < 2) return fail(BSSN_ERR_INVALID, std::string(where) + ": margin must be at least 2");
    G.cs = cs;
    return BSSN_OK;
}

int sphere_ok(int nt, int np, const char* where) {
    if (nt < 6 || np < 6 || np % 2)
        return fail(BSSN_ERR_INVALID, std::string(where) + ": use at least six nodes per angle and an even n_phi");
    if ((long long)nt * np > (1 << 22)) return fail(BSSN_ERR_INVALID, std::string(where) + ": surface too large");
    return BSSN_OK;
}

Band band_of(void* ws, int nt, int np) {
    Band B;
    B.n = nt * np;
    B.kl = std::min(3 * np - 1, B.n - 1);
    B.ku2 = std::min(2 * B.kl, B.n - 1);
    B.ld = B.kl + B.ku2 + 1;
    B.a = static_cast<double*>(ws);
    return B;
}

size_t band_bytes(int nt, int np) {
    const Band B = band_of(nullptr, nt, np);
    return (size_t)B.n * B.ld * sizeof(double);
}

// Workspace of the Newton direction: the band, then the pivots (U's
// diagonal), the right-hand side / solution, its two-number summary and the
// nodes' bad flags.
struct Factor {
    Band B;
    double *diag, *rhs, *sum;
    int *bad, *piv;
    double* panel[2];  // double-buffered copies of the next panel (blocked form)
};

size_t panel_doubles(const Band& B) { return (size_t)kPanel * (B.kl + kPanel); }

Factor factor_of(void* ws, int nt, int np) {
    Factor F;
    F.B = band_of(ws, nt, np);
    char* rest = static_cast<char*>(ws) + band_bytes(nt, np);
    F.diag = reinterpret_cast<double*>(rest);
    F.rhs = F.diag + F.B.n;
    F.sum = F.rhs + F.B.n;
    F.bad = reinterpret_cast<int*>(F.sum + 2);
    F.piv = F.bad + F.B.n;
    const size_t off = ((size_t)(reinterpret_cast<char*>(F.piv + F.B.n) - static_cast<char*>(ws)) + 15) & ~(size_t)15;
    F.panel[0] = reinterpret_cast<double*>(static_cast<char*>(ws) + off);
    F.panel[1] = F.panel[0] + panel_doubles(F.B);
    return F;
}

// Launch with the programmatic-stream-serialisation attribute (dependent
// launch), counted and timed like every other launch.
template <typename... P, typename... A>
cudaError_t launch_dependent(void (*kernel)(P...), unsigned blocks, unsigned threads, size_t smem, cudaStream_t s,
                             A... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(blocks);
    cfg.blockDim = dim3(threads);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    prof_begin(KC_HORIZON_SOLVE, s);
    const cudaError_t e = cudaLaunchKernelEx(&cfg, kernel, args...);
    prof_end(KC_HORIZON_SOLVE, s);
    return e;
}

// The dynamic shared-memory opt-in of k_band_back_shared is an attribute of
// the kernel in the current device's context, so it is set once per device
// (under a lock: several host threads may solve at once).
cudaError_t configure_back_shared() {
    static std::mutex lock;
    static std::set<int> configured;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    std::lock_guard<std::mutex> guard(lock);
    if (configured.count(dev)) return cudaSuccess;
    e = cudaFuncSetAttribute(k_band_back_shared, cudaFuncAttributeMaxDynamicSharedMemorySize, kBackSmemMax);
    if (e == cudaSuccess) configured.insert(dev);
    return e;
}

// The factorisation and back substitution: one launch per band column, then
// one for the back substitution, each a dependent launch of the one before.
// Returns the number of launches; *err receives the first launch error.
int enqueue_factor(const Factor& F, cudaStream_t s, cudaError_t* err) {
    const Band& B = F.B;
    cudaError_t first = cudaSuccess;
    auto keep = [&first](cudaError_t e) { if (first == cudaSuccess) first = e; };
    const bool fused = B.kl + 2 <= 32 * kRowsPerLane;
    const bool blocked = B.kl + kPanel <= kPanelRows;
    int launches = 0;
    if (blocked) {
        const int P = B.kl + kPanel;
        BSSN_LAUNCH(KC_HORIZON_SOLVE, k_panel_init, (kPanel * P + 255) / 256, 256, s, B, F.panel[0]);
        ++launches;
        for (int c0 = 0, p = 0; c0 < B.n; c0 += kPanel, ++p) {
            const int ncol = std::min(kPanel, B.n - c0);
            const int first = c0 + ncol;
            const int lastc = std::min(B.n - 1, c0 + ncol - 1 + B.ku2);
            const int ntrail = lastc >= first ? lastc - first + 1 : 0;
            const unsigned blocks = (unsigned)((ntrail + 1 + kPanelWarps - 1) / kPanelWarps);
            keep(launch_dependent(k_band_panel, blocks, kPanelWarps * 32, 0, s, B, c0,
                                  (const double*)F.panel[p % 2], F.panel[(p + 1) % 2], F.rhs, F.diag));
            ++launches;
        }
    }
    for (int k = 0; !blocked && k < B.n; ++k) {
        const int cols = std::min(B.n - 1, k + B.ku2) - k + 1;  // trailing columns plus the right-hand side
        const unsigned blocks = (unsigned)((cols + kStepWarps - 1) / kStepWarps);
        if (fused)
            keep(launch_dependent(k_band_step_fused, blocks, kStepWarps * 32, 0, s, B, k, k == 0 ? 1 : 0, F.rhs,
                                  F.diag, F.piv));
        else
            keep(launch_dependent(k_band_step, blocks, kStepWarps * 32, 0, s, B, k, F.rhs, F.diag));
        ++launches;
    }
    const size_t smem = 2 * (size_t)B.n * sizeof(double);
    if (smem <= (size_t)kBackSmemMax && B.ku2 <= kBackThreads) {
        keep(configure_back_shared());
        keep(launch_dependent(k_band_back_shared, 1, kBackThreads, smem, s, B, F.rhs, F.diag, F.sum));
    } else {
        keep(launch_dependent(k_band_back, 1, kBackThreads, 0, s, B, F.rhs, F.diag, F.sum));
    }
    if (err) *err = first;
    return launches + 1;
}

// Instantiated factorisation graphs per thread, keyed by device, workspace
// and surface shape (the kernels' pointers all live in the workspace).
struct FactorGraphs {
    cudaStream_t capture = nullptr;
    std::map<std::tuple<int, void*, int, int>, cudaGraphExec_t> execs;
    std::map<std::tuple<int, void*, int, int>, int> launches;
};

cudaError_t factor_graph(const Factor& F, void* ws, int nt, int np, cudaGraphExec_t& out, int& launches) {
    thread_local FactorGraphs graphs;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    const auto key = std::make_tuple(dev, ws, nt, np);
    auto it = graphs.execs.find(key);
    if (it != graphs.execs.end()) {
        out = it->second;
        launches = graphs.launches[key];
        return cudaSuccess;
    }
    if (graphs.execs.size() >= 16) {
        for (auto& kv : graphs.execs) cudaGraphExecDestroy(kv.second);
        graphs.execs.clear();
        graphs.launches.clear();
    }
    if (!graphs.capture) {
        e = cudaStreamCreateWithFlags(&graphs.capture, cudaStreamNonBlocking);
        if (e != cudaSuccess) return e;
    }
    e = configure_back_shared();
    if (e != cudaSuccess) return e;
    e = cudaStreamBeginCapture(graphs.capture, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return e;
    cudaError_t launched = cudaSuccess;
    const int recorded = enqueue_factor(F, graphs.capture, &launched);
    count_launches(-recorded);  // recorded, not run
    graphs.launches[key] = recorded;
    cudaGraph_t graph = nullptr;
    e = cudaStreamEndCapture(graphs.capture, &graph);
    if (e == cudaSuccess && launched != cudaSuccess) e = launched;
    cudaGraphExec_t exec = nullptr;
    if (e == cudaSuccess) e = cudaGraphInstantiate(&exec, graph, 0);
    if (graph) cudaGraphDestroy(graph);
    if (e != cudaSuccess) {
        graphs.launches.erase(key);
        return e;
    }
    graphs.execs[key] = exec;
    out = exec;
    launches = graphs.launches[key];
    return cudaSuccess;
}

int assemble(const HGeom& G, const double center[3], const double* radius, int nt, int np, double fd_step,
             const Band& B, double* expansion, int* bad, cudaStream_t s) {
    Sphere S{nt, np, radius, nullptr, 0.0};
    cudaError_t e = cudaMemsetAsync(B.a, 0, (size_t)B.n * B.ld * sizeof(double), s);
    if (e != cudaSuccess) return cuda_status(e, "bssn_horizon: band clear");
    const unsigned blocks = (unsigned)((B.n + kSurfWarps - 1) / kSurfWarps);
    BSSN_LAUNCH(KC_HORIZON_SURFACE, k_surface, blocks, kSurfWarps * 32, s, G, S, center[0], center[1], center[2],
                (double*)nullptr, expansion, (double*)nullptr, bad, B, fd_step);
    return cuda_status(cudaGetLastError(), "bssn_horizon: jacobian");
}

}  // namespace
}  // namespace bssn

using namespace bssn;

extern "C" int bssn_horizon_sample(const BssnHorizonGeometry* geometry, const double* points, int64_t npoints,
                                   double* gamma, double* d_gamma, double* curvature, int32_t* valid,
                                   void* stream) {
    HGeom G;
    int st = geometry_of(geometry, G, "bssn_horizon_sample");
    if (st != BSSN_OK) return st;
    if (npoints < 0 || (npoints > 0 && !points)) return fail(BSSN_ERR_INVALID, "bssn_horizon_sample: bad points");
    if (npoints == 0) return BSSN_OK;
    const unsigned blocks = (unsigned)((npoints + kHThreads - 1) / kHThreads);
    BSSN_LAUNCH(KC_HORIZON_SURFACE, k_sample, blocks, kHThreads, (cudaStream_t)stream, G, points, (long long)npoints,
                gamma, d_gamma, curvature, valid);
    return cuda_status(cudaGetLastError(), "bssn_horizon_sample");
}

extern "C" int bssn_horizon_angular_derivatives(const double* radius, int32_t n_theta, int32_t n_phi, double* out,
                                                void* stream) {
    int st = sphere_ok(n_theta, n_phi, "bssn_horizon_angular_derivatives");
    if (st != BSSN_OK) return st;
    if (!radius || !out) return fail(BSSN_ERR_INVALID, "bssn_horizon_angular_derivatives: null pointer");
    Sphere S{n_theta, n_phi, radius, nullptr, 0.0};
    const int n = n_theta * n_phi;
    BSSN_LAUNCH(KC_HORIZON_SURFACE, k_ang, (n + kHThreads - 1) / kHThreads, kHThreads, (cudaStream_t)stream, S, out);
    return cuda_status(cudaGetLastError(), "bssn_horizon_angular_derivatives");
}

extern "C" size_t bssn_horizon_workspace_bytes(int32_t n_theta, int32_t n_phi) {
    if (n_theta < 6 || n_phi < 6 || n_phi % 2 || (long long)n_theta * n_phi > (1 << 22)) return 0;
    const size_t n = (size_t)n_theta * n_phi;
    return band_bytes(n_theta, n_phi) + 2 * n * sizeof(double) + 2 * sizeof(double) + 2 * n * sizeof(int) + 16 +
           2 * panel_doubles(band_of(nullptr, n_theta, n_phi)) * sizeof(double);
}

extern "C" int bssn_horizon_surface(const BssnHorizonGeometry* geometry, const double center[3],
                                    const double* radius, const double* direction, double step, int32_t n_theta,
                                    int32_t n_phi, const double* area_weights, double* trial, double* expansion,
                                    double* density, double* summary, void* workspace, size_t workspace_bytes,
                                    void* stream) {
    HGeom G;
    int st = geometry_of(geometry, G, "bssn_horizon_surface");
    if (st != BSSN_OK) return st;
    if ((st = sphere_ok(n_theta, n_phi, "bssn_horizon_surface")) != BSSN_OK) return st;
    if (!center || !radius || !expansion || !summary)
        return fail(BSSN_ERR_INVALID, "bssn_horizon_surface: null pointer");
    const int n = n_theta * n_phi;
    if (!workspace || workspace_bytes < (size_t)n * sizeof(int))
        return fail(BSSN_ERR_WORKSPACE, "bssn_horizon_surface: workspace too small");
    if (direction && !trial) return fail(BSSN_ERR_INVALID, "bssn_horizon_surface: a direction needs a trial buffer");
    cudaStream_t s = (cudaStream_t)stream;
    int* bad = static_cast<int*>(workspace);
    Sphere S{n_theta, n_phi, radius, direction, step};
    Band none{nullptr, 0, 0, 0, 0};
    BSSN_LAUNCH(KC_HORIZON_SURFACE, k_surface, (n + kSurfWarps - 1) / kSurfWarps, kSurfWarps * 32, s, G, S, center[0],
                center[1], center[2], trial, expansion, density, bad, none, 0.0);
    BSSN_LAUNCH(KC_HORIZON_SURFACE, k_surface_summary, 1, kSumThreads, s, direction ? (const double*)trial : radius,
                expansion, density, bad, area_weights, n_theta, n_phi, summary);
    return cuda_status(cudaGetLastError(), "bssn_horizon_surface");
}

extern "C" int bssn_horizon_jacobian(const BssnHorizonGeometry* geometry, const double center[3],
                                     const double* radius, int32_t n_theta, int32_t n_phi, double fd_step,
                                     double* dense, void* workspace, size_t workspace_bytes, void* stream) {
    HGeom G;
    int st = geometry_of(geometry, G, "bssn_horizon_jacobian");
    if (st != BSSN_OK) return st;
    if ((st = sphere_ok(n_theta, n_phi, "bssn_horizon_jacobian")) != BSSN_OK) return st;
    if (!center || !radius || !dense) return fail(BSSN_ERR_INVALID, "bssn_horizon_jacobian: null pointer");
    if (!workspace || workspace_bytes < bssn_horizon_workspace_bytes(n_theta, n_phi))
        return fail(BSSN_ERR_WORKSPACE, "bssn_horizon_jacobian: workspace too small");
    cudaStream_t s = (cudaStream_t)stream;
    const Factor F = factor_of(workspace, n_theta, n_phi);
    if ((st = assemble(G, center, radius, n_theta, n_phi, fd_step, F.B, F.rhs, F.bad, s)) != BSSN_OK) return st;
    const long long total = (long long)F.B.n * F.B.n;
    BSSN_LAUNCH(KC_HORIZON_SOLVE, k_band_dense, (unsigned)((total + 255) / 256), 256, s, F.B, dense);
    return cuda_status(cudaGetLastError(), "bssn_horizon_jacobian");
}

extern "C" int bssn_horizon_newton_direction(const BssnHorizonGeometry* geometry, const double center[3],
                                             const double* radius, const double* expansion, int32_t n_theta,
                                             int32_t n_phi, double fd_step, double* delta, double* summary,
                                             void* workspace, size_t workspace_bytes, void* stream) {
    HGeom G;
    int st = geometry_of(geometry, G, "bssn_horizon_newton_direction");
    if (st != BSSN_OK) return st;
    if ((st = sphere_ok(n_theta, n_phi, "bssn_horizon_newton_direction")) != BSSN_OK) return st;
    if (!center || !radius || !expansion || !delta || !summary)
        return fail(BSSN_ERR_INVALID, "bssn_horizon_newton_direction: null pointer");
    if (!workspace || workspace_bytes < bssn_horizon_workspace_bytes(n_theta, n_phi))
        return fail(BSSN_ERR_WORKSPACE, "bssn_horizon_newton_direction: workspace too small");
    cudaStream_t s = (cudaStream_t)stream;
    const Factor F = factor_of(workspace, n_theta, n_phi);
    // the assembly's own expansion lands in rhs, which -Theta then replaces
    if ((st = assemble(G, center, radius, n_theta, n_phi, fd_step, F.B, F.rhs, F.bad, s)) != BSSN_OK) return st;
    BSSN_LAUNCH(KC_HORIZON_SOLVE, k_negate, (F.B.n + 255) / 256, 256, s, expansion, F.rhs, F.B.n);
    cudaError_t e = cudaSuccess;
    cudaGraphExec_t exec = nullptr;
    int launches = 0;
    // Replay the factorisation's launches as a CUDA graph unless per-kernel
    // profiling is on (which times every launch with events of its own).
    if (!profiling_enabled()) e = factor_graph(F, workspace, n_theta, n_phi, exec, launches);
    if (e != cudaSuccess) return cuda_status(e, "bssn_horizon_newton_direction (graph capture)");
    if (exec) {
        count_launches(launches);
        e = cudaGraphLaunch(exec, s);
    } else {
        enqueue_factor(F, s, &e);
        if (e == cudaSuccess) e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(delta, F.rhs, (size_t)F.B.n * sizeof(double), cudaMemcpyDeviceToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(summary, F.sum, 2 * sizeof(double), cudaMemcpyDeviceToDevice, s);
    return cuda_status(e, "bssn_horizon_newton_direction");
}

extern "C" int bssn_horizon_regrid(const double* radius, int32_t n_theta, int32_t n_phi, const double* theta,
                                   int32_t n_theta_out, const double* phi, int32_t n_phi_out, double* out,
                                   void* stream) {
    int st = sphere_ok(n_theta, n_phi, "bssn_horizon_regrid");
    if (st != BSSN_OK) return st;
    if (n_theta_out < 1 || n_phi_out < 1 || (long long)n_theta_out * n_phi_out > (1 << 24))
        return fail(BSSN_ERR_INVALID, "bssn_horizon_regrid: bad output grid");
    if (!radius || !theta || !phi || !out) return fail(BSSN_ERR_INVALID, "bssn_horizon_regrid: null pointer");
    const int n = n_theta_out * n_phi_out;
    BSSN_LAUNCH(KC_HORIZON_SURFACE, k_regrid, (n + kHThreads - 1) / kHThreads, kHThreads, (cudaStream_t)stream,
                radius, n_theta, n_phi, theta, n_theta_out, phi, n_phi_out, out);
    return cuda_status(cudaGetLastError(), "bssn_horizon_regrid");
}
