// BSSN right-hand side on a padded patch (sm_103a, FP64).
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
//   k_rhs_kgt        dt K, dt Gt^i (JAX_BSSN/bssn/extrinsic_curvature.py:31-92,
//                    conformal_connection.py:19-162)
//   k_rhs_at         dt At_ij incl. W^2 R_ij, W^2 D_i D_j alpha
//                    (JAX_BSSN/bssn/extrinsic_curvature.py:119-224, geometry.py:21-186)
//   k_mom_*          kappa != 0 only: M_i, d_l M_i and the constraint-damping
//                    term (JAX_BSSN/bssn/constraints.py:22-213)
//   k_sommerfeld     radial Sommerfeld replacement on active owned faces
//                    (JAX_BSSN/evolution/boundaries.py:150-171)
// Operators commute along different axes, so each mixed derivative is formed
// once (outer axis = the larger index) and used for both orderings.
#include "bssn_fields.cuh"
#include "bssn_kernels.h"
#include "bssn_profile.h"

namespace bssn {

constexpr int kThreads = 128;

__device__ __forceinline__ bool in_range(const Axis& a, int i) { return i >= a.lo && i < a.hi; }

// ---------------------------------------------------------------------------
// inner first derivatives
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kThreads)
k_first_derivs(const double* __restrict__ u, const double* __restrict__ der,
               double* __restrict__ d1, Geo G, Box ext, int with_mom) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= ext.count) return;
    int ix[3];
    ext.coords(t, ix);
    const long long p = lin(G, ix);
    const long long cs = G.cs;
    const int nfield = with_mom ? NMIX + NMIX_MOM : NMIX;
#pragma unroll 1
    for (int d = 0; d < 3; ++d) {
        if (!in_range(G.ax[d], ix[d])) continue;
#pragma unroll 1
        for (int f = 0; f < NMIX; ++f)
            d1[((long long)(d * nfield + f)) * cs + p] = D1(u + mix_source(f) * cs + p, G, d, ix[d]);
        if (with_mom) {
#pragma unroll 1
            for (int f = 0; f < 7; ++f)  // At (6), K
                d1[((long long)(d * nfield + NMIX + f)) * cs + p] = D1(u + (AXX + f) * cs + p, G, d, ix[d]);
#pragma unroll 1
            for (int f = 0; f < 9; ++f)  // B_i^j from the derived buffer (slots 6..14)
                d1[((long long)(d * nfield + NMIX + 7 + f)) * cs + p] = D1(der + (6 + f) * cs + p, G, d, ix[d]);
        }
    }
}

struct PointCtx {
    int ix[3];
    long long p;
};

__device__ __forceinline__ bool point(const Box& B, PointCtx& c, const Geo& G) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= B.count) return false;
    B.coords(t, c.ix);
    c.p = lin(G, c.ix);
    return true;
}

// d1 buffer accessor: first derivative along d of stored field f.
__device__ __forceinline__ const double* d1ptr(const double* d1, const Geo& G, int nfield, int d, int f,
                                               long long p) {
    return d1 + ((long long)(d * nfield + f)) * G.cs + p;
}

// Mixed second derivative d_m d_n of stored field f (m != n): outer axis is
// max(m,n), inner axis min(m,n).
__device__ __forceinline__ double mixed(const double* d1, const Geo& G, int nfield, int f, int m, int n,
                                        const PointCtx& c) {
    const int inner = m < n ? m : n;
    const int outer = m < n ? n : m;
    return D1(d1ptr(d1, G, nfield, inner, f, c.p), G, outer, c.ix[outer]);
}

// Symmetric Hessian of stored field f whose state component is comp:
// h[sym(i,j)] = d_i d_j f, D2 on the diagonal.
__device__ __forceinline__ void hessian(const double* __restrict__ u, const double* d1, const Geo& G,
                                        int nfield, int comp, int f, const PointCtx& c, double (&h)[6]) {
    const double* fp = u + comp * G.cs + c.p;
    h[0] = D2(fp, G, 0, c.ix[0]);
    h[3] = D2(fp, G, 1, c.ix[1]);
    h[5] = D2(fp, G, 2, c.ix[2]);
    h[1] = mixed(d1, G, nfield, f, 0, 1, c);
    h[2] = mixed(d1, G, nfield, f, 0, 2, c);
    h[4] = mixed(d1, G, nfield, f, 1, 2, c);
}

__device__ __forceinline__ double contract_sym(const double (&a)[6], const double (&b)[6]) {
    return a[0] * b[0] + a[3] * b[3] + a[5] * b[5] + 2.0 * (a[1] * b[1] + a[2] * b[2] + a[4] * b[4]);
}

// W^2 D_i D_j alpha (JAX_BSSN/bssn/geometry.py:122-186)
__device__ __forceinline__ void w2_lapse_hessian(const double* __restrict__ u, const double* d1,
                                                 const Geo& G, int nfield, const PointCtx& c,
                                                 const double (&g)[6], const double (&gi)[6],
                                                 const double (&c2)[3][6], const double (&dW)[3],
                                                 const double (&da)[3], double W, double (&out)[6]) {
    double h[6];
    hessian(u, d1, G, nfield, CALPHA, MIX_ALPHA, c, h);
    double gw = 0.0;
#pragma unroll
    for (int m = 0; m < 3; ++m)
#pragma unroll
        for (int n = 0; n < 3; ++n) gw += gi[sym(m, n)] * dW[m] * da[n];
    const double W2 = W * W;
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = i; j < 3; ++j) {
            const int s = sym(i, j);
            const double conf = h[s] - (c2[0][s] * da[0] + c2[1][s] * da[1] + c2[2][s] * da[2]);
            const double grad = dW[i] * da[j] + dW[j] * da[i] - g[s] * gw;
            out[s] = W2 * conf + W * grad;
        }
}

__device__ __forceinline__ void load_sym(const double* __restrict__ u, int base, const Geo& G, long long p,
                                         double (&v)[6]) {
#pragma unroll
    for (int s = 0; s < 6; ++s) v[s] = u[(base + s) * G.cs + p];
}

__device__ __forceinline__ void load_metric_derivs(const double* d1, const Geo& G, int nfield, long long p,
                                                   double (&dg)[3][6]) {
#pragma unroll
    for (int k = 0; k < 3; ++k)
#pragma unroll
        for (int s = 0; s < 6; ++s) dg[k][s] = d1ptr(d1, G, nfield, k, MIX_G + s, p)[0];
}

// W^2 R_ij without inverse powers of W (JAX_BSSN/bssn/geometry.py:21-119).
__device__ __forceinline__ void w2_ricci(const double* __restrict__ u, const double* d1, const Geo& G,
                                         int nfield, const PointCtx& c, const double (&g)[6],
                                         const double (&gi)[6], const double (&c1)[3][6],
                                         const double (&c2)[3][6], const double (&dW)[3], double W,
                                         double (&w2r)[6]) {
    const long long cs = G.cs, p = c.p;
    // --- conformal Ricci tensor (geometry.py:44-81) ---
    double ric[6];
#pragma unroll 1
    for (int s = 0; s < 6; ++s) {
        double h[6];
        hessian(u, d1, G, nfield, GXX + s, MIX_G + s, c, h);
        ric[s] = -0.5 * contract_sym(gi, h);
    }
    {
        const double Gt[3] = {u[GTX * cs + p], u[GTY * cs + p], u[GTZ * cs + p]};
        double dG[3][3];  // dG[d][i] = d_d Gt^i
#pragma unroll 1
        for (int d = 0; d < 3; ++d)
#pragma unroll 1
            for (int i = 0; i < 3; ++i) dG[d][i] = D1(u + (GTX + i) * cs + p, G, d, c.ix[d]);
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int j = i; j < 3; ++j) {
                double t2 = 0.0, t3 = 0.0;
#pragma unroll
                for (int m = 0; m < 3; ++m) {
                    t2 += g[sym(m, i)] * dG[j][m] + g[sym(m, j)] * dG[i][m];
                    t3 += Gt[m] * (c1[i][sym(j, m)] + c1[j][sym(i, m)]);
                }
                ric[sym(i, j)] += 0.5 * t2 + 0.5 * t3;
            }
    }
    // term4 + term5: loop over k to bound live registers.
#pragma unroll 1
    for (int kk = 0; kk < 3; ++kk) {
        double X[3][3], Y[3][3];  // X[n][i] = g^mn Gamma^k_mi ; Y[m][j] = g^mn Gamma_kjn
#pragma unroll
        for (int a = 0; a < 3; ++a)
#pragma unroll
            for (int b = 0; b < 3; ++b) {
                X[a][b] = gi[sym(0, a)] * c2[kk][sym(0, b)] + gi[sym(1, a)] * c2[kk][sym(1, b)]
                          + gi[sym(2, a)] * c2[kk][sym(2, b)];
                Y[a][b] = gi[sym(a, 0)] * c1[kk][sym(b, 0)] + gi[sym(a, 1)] * c1[kk][sym(b, 1)]
                          + gi[sym(a, 2)] * c1[kk][sym(b, 2)];
            }
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int j = i; j < 3; ++j) {
                double t4 = 0.0, t5 = 0.0;
#pragma unroll
                for (int n = 0; n < 3; ++n) {
                    // term4: g^mn Gamma^k_mi Gamma_jkn + (i<->j); c1[j][sym(k,n)] = Gamma_jkn
                    t4 += X[n][i] * c1[j][sym(kk, n)] + X[n][j] * c1[i][sym(kk, n)];
                    // term5: Gamma^k_im g^mn Gamma_kjn
                    t5 += c2[kk][sym(i, n)] * Y[n][j];
                }
                ric[sym(i, j)] += t4 + t5;
            }
    }
    // --- W terms: W (D_i D_j W + gt_ij lap W) - 2 gt_ij |dW|^2 (geometry.py:84-117) ---
    {
        double hW[6];
        hessian(u, d1, G, nfield, CW, MIX_W, c, hW);
#pragma unroll
        for (int s = 0; s < 6; ++s) hW[s] -= c2[0][s] * dW[0] + c2[1][s] * dW[1] + c2[2][s] * dW[2];
        const double lap = contract_sym(gi, hW);
        double grad2 = 0.0;
#pragma unroll
        for (int m = 0; m < 3; ++m)
#pragma unroll
            for (int n = 0; n < 3; ++n) grad2 += gi[sym(m, n)] * dW[m] * dW[n];
        const double W2 = W * W;
#pragma unroll
        for (int s = 0; s < 6; ++s) w2r[s] = W2 * ric[s] + (W * (hW[s] + g[s] * lap) - 2.0 * g[s] * grad2);
    }
}

// ---------------------------------------------------------------------------
// dt gt_ij, dt W, dt alpha, dt beta^i
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kThreads)
k_rhs_gauge(const double* __restrict__ u, const double* __restrict__ d1, double* __restrict__ k,
            Geo G, Box B, int nfield) {
    PointCtx c;
    if (!point(B, c, G)) return;
    const long long cs = G.cs, p = c.p;
    const double beta[3] = {u[BX * cs + p], u[BY * cs + p], u[BZ * cs + p]};
    double db[3][3];  // db[i][j] = d_j beta^i
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) db[i][j] = d1ptr(d1, G, nfield, j, MIX_B + i, p)[0];
    const double div = db[0][0] + db[1][1] + db[2][2];
    const double alpha = u[CALPHA * cs + p];
    const double K = u[CK * cs + p];
    const double W = u[CW * cs + p];
    double g[6];
    load_sym(u, GXX, G, p, g);

#pragma unroll 1
    for (int s = 0; s < 6; ++s) {
        const int i = s < 3 ? 0 : (s < 5 ? 1 : 2);
        const int j = s < 3 ? s : (s < 5 ? s - 2 : 2);
        const double* f = u + (GXX + s) * cs + p;
        double lie = 0.0;
#pragma unroll
        for (int m = 0; m < 3; ++m) lie += g[sym(m, i)] * db[m][j] + g[sym(m, j)] * db[m][i];
        const double v = ADV(f, G, c.ix, beta) + lie + (-2.0 / 3.0) * g[s] * div
                         + (-2.0) * alpha * u[(AXX + s) * cs + p];
        k[(GXX + s) * cs + p] = v + KO(f, G, c.ix);
    }
    {
        const double* f = u + CW * cs + p;
        const double v = ADV(f, G, c.ix, beta) + (1.0 / 3.0) * alpha * W * K - (1.0 / 3.0) * W * div;
        k[CW * cs + p] = v + KO(f, G, c.ix);
    }
    {
        const double* f = u + CALPHA * cs + p;
        const double slicing = (G.gauge == 0) ? -(alpha * alpha) * K : -2.0 * alpha * K;
        k[CALPHA * cs + p] = slicing + ADV(f, G, c.ix, beta) + KO(f, G, c.ix);
    }
#pragma unroll 1
    for (int i = 0; i < 3; ++i) {
        const double* f = u + (BX + i) * cs + p;
        double v;
        if (G.zero_shift) {
            v = 0.0 * beta[i];
        } else {
            v = G.g * u[(GTX + i) * cs + p] + ADV(f, G, c.ix, beta) + (-G.eta) * beta[i];
            v = v + KO(f, G, c.ix);
        }
        k[(BX + i) * cs + p] = v;
    }
}

// ---------------------------------------------------------------------------
// dt K and dt Gt^i
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kThreads)
k_rhs_kgt(const double* __restrict__ u, const double* __restrict__ d1, double* __restrict__ k,
          Geo G, Box B, int nfield) {
    PointCtx c;
    if (!point(B, c, G)) return;
    const long long cs = G.cs, p = c.p;
    double g[6], gi[6];
    load_sym(u, GXX, G, p, g);
    inverse_metric(g, gi);
    double c1[3][6], c2[3][6];
    {
        double dg[3][6];
        load_metric_derivs(d1, G, nfield, p, dg);
        christoffel(dg, gi, c1, c2);
    }
    double dW[3], da[3], dK[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        dW[d] = d1ptr(d1, G, nfield, d, MIX_W, p)[0];
        da[d] = d1ptr(d1, G, nfield, d, MIX_ALPHA, p)[0];
        dK[d] = D1(u + CK * cs + p, G, d, c.ix[d]);
    }
    const double W = u[CW * cs + p];
    const double alpha = u[CALPHA * cs + p];
    const double K = u[CK * cs + p];
    const double beta[3] = {u[BX * cs + p], u[BY * cs + p], u[BZ * cs + p]};
    double A[6];
    load_sym(u, AXX, G, p, A);
    double Au[6];  // A^ij = g^ik g^jl A_kl
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

    // dt K
    {
        double h[6];
        w2_lapse_hessian(u, d1, G, nfield, c, g, gi, c2, dW, da, W, h);
        const double first = -contract_sym(gi, h);
        const double second = alpha * contract_sym(A, Au);
        const double third = alpha * (K * K) / 3.0;
        const double* f = u + CK * cs + p;
        k[CK * cs + p] = first + second + third + ADV(f, G, c.ix, beta) + KO(f, G, c.ix);
    }

    // dt Gt^i
    double db[3][3];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) db[i][j] = d1ptr(d1, G, nfield, j, MIX_B + i, p)[0];
    const double div = db[0][0] + db[1][1] + db[2][2];
    const double Wf = fmax(W, 1.0e-12);
    double hb[3][6];  // hb[i][sym(m,n)] = d_m d_n beta^i
#pragma unroll 1
    for (int i = 0; i < 3; ++i) hessian(u, d1, G, nfield, BX + i, MIX_B + i, c, hb[i]);
    double graddiv[3];
#pragma unroll
    for (int m = 0; m < 3; ++m) graddiv[m] = hb[0][sym(m, 0)] + hb[1][sym(m, 1)] + hb[2][sym(m, 2)];
    const double Gt[3] = {u[GTX * cs + p], u[GTY * cs + p], u[GTZ * cs + p]};
#pragma unroll 1
    for (int i = 0; i < 3; ++i) {
        double t1 = 0.0, t3 = 0.0, t4 = 0.0, t7 = 0.0, t9 = 0.0;
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            t1 += gi[sym(i, j)] * dK[j];
            t3 += Au[sym(i, j)] * dW[j];
            t4 += Au[sym(i, j)] * da[j];
            t7 += Gt[j] * db[i][j];
            t9 += gi[sym(i, j)] * graddiv[j];
        }
        const double t2 = contract_sym(c2[i], Au);
        const double t8 = contract_sym(gi, hb[i]);
        const double* f = u + (GTX + i) * cs + p;
        const double v = (-4.0 / 3.0) * alpha * t1 + 2.0 * alpha * t2 + (-6.0 * alpha / Wf) * t3
                         - 2.0 * t4 + ADV(f, G, c.ix, beta) + (2.0 / 3.0) * Gt[i] * div - t7 + t8
                         + (1.0 / 3.0) * t9;
        k[(GTX + i) * cs + p] = v + KO(f, G, c.ix);
    }
}

// ---------------------------------------------------------------------------
// dt At_ij
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kThreads)
k_rhs_at(const double* __restrict__ u, const double* __restrict__ d1, const double* __restrict__ damp,
         double* __restrict__ k, Geo G, Box B, int nfield) {
    PointCtx c;
    if (!point(B, c, G)) return;
    const long long cs = G.cs, p = c.p;
    double g[6], gi[6];
    load_sym(u, GXX, G, p, g);
    inverse_metric(g, gi);
    double c1[3][6], c2[3][6];
    {
        double dg[3][6];
        load_metric_derivs(d1, G, nfield, p, dg);
        christoffel(dg, gi, c1, c2);
    }
    double dW[3], da[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        dW[d] = d1ptr(d1, G, nfield, d, MIX_W, p)[0];
        da[d] = d1ptr(d1, G, nfield, d, MIX_ALPHA, p)[0];
    }
    const double W = u[CW * cs + p];
    const double alpha = u[CALPHA * cs + p];

    double w2r[6];
    w2_ricci(u, d1, G, nfield, c, g, gi, c1, c2, dW, W, w2r);
    // --- [alpha W^2 R_ij - W^2 D_i D_j alpha]^TF ---
    double T[6];
    {
        double h[6];
        w2_lapse_hessian(u, d1, G, nfield, c, g, gi, c2, dW, da, W, h);
#pragma unroll
        for (int s = 0; s < 6; ++s) T[s] = alpha * w2r[s] - h[s];
        const double tr = contract_sym(gi, T);
#pragma unroll
        for (int s = 0; s < 6; ++s) T[s] = T[s] - (1.0 / 3.0) * g[s] * tr;
    }
    // --- remaining terms ---
    const double K = u[CK * cs + p];
    double A[6];
    load_sym(u, AXX, G, p, A);
    const double beta[3] = {u[BX * cs + p], u[BY * cs + p], u[BZ * cs + p]};
    double db[3][3];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) db[i][j] = d1ptr(d1, G, nfield, j, MIX_B + i, p)[0];
    const double div = db[0][0] + db[1][1] + db[2][2];
#pragma unroll 1
    for (int s = 0; s < 6; ++s) {
        const int i = s < 3 ? 0 : (s < 5 ? 1 : 2);
        const double* f = u + (AXX + s) * cs + p;
        const int j = s < 3 ? s : (s < 5 ? s - 2 : 2);
        double AgA = 0.0, lie = 0.0;
#pragma unroll
        for (int kk = 0; kk < 3; ++kk) {
#pragma unroll
            for (int l = 0; l < 3; ++l) AgA += A[sym(i, kk)] * gi[sym(kk, l)] * A[sym(l, j)];
            lie += A[sym(kk, i)] * db[kk][j] + A[sym(kk, j)] * db[kk][i];
        }
        double v = alpha * K * A[s] - 2.0 * alpha * AgA + T[s] + ADV(f, G, c.ix, beta) + lie
                   + (-2.0 / 3.0) * A[s] * div;
        if (damp != nullptr) v += damp[s * cs + p];
        k[(AXX + s) * cs + p] = v + KO(f, G, c.ix);
    }
}

// ---------------------------------------------------------------------------
// kappa != 0: derived fields on the whole patch (constraints.py:112-118):
//   der[0..5]  = gt^ij        der[6..14] = B_i^j = gt^jk At_ik
//   der[15..23]= B_i^j / max(W, 1e-12)
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kThreads)
k_mom_derived(const double* __restrict__ u, double* __restrict__ der, Geo G, Box all) {
    PointCtx c;
    if (!point(all, c, G)) return;
    const long long cs = G.cs, p = c.p;
    double g[6], gi[6], A[6];
    load_sym(u, GXX, G, p, g);
    load_sym(u, AXX, G, p, A);
    inverse_metric(g, gi);
    const double Wf = fmax(u[CW * cs + p], 1.0e-12);
#pragma unroll
    for (int s = 0; s < 6; ++s) der[s * cs + p] = gi[s];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            const double b = gi[sym(j, 0)] * A[sym(i, 0)] + gi[sym(j, 1)] * A[sym(i, 1)] + gi[sym(j, 2)] * A[sym(i, 2)];
            der[(6 + 3 * i + j) * cs + p] = b;
            der[(15 + 3 * i + j) * cs + p] = b / Wf;
        }
}

// kappa/2 alpha (D_j M_i + D_i M_j) into damp[6] (extrinsic_curvature.py:390-404)
__global__ void __launch_bounds__(kThreads)
k_mom_damping(const double* __restrict__ u, const double* __restrict__ der, const double* __restrict__ d1,
              double* __restrict__ damp, Geo G, Box B, int nfield) {
    PointCtx c;
    if (!point(B, c, G)) return;
    const long long cs = G.cs, p = c.p;
    const int fA = NMIX, fK = NMIX + 6, fB = NMIX + 7;
    double gi[6];
#pragma unroll
    for (int s = 0; s < 6; ++s) gi[s] = der[s * cs + p];
    const double W = u[CW * cs + p];
    const double Wf = fmax(W, 1.0e-12);
    double dW[3], dK[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        dW[d] = d1ptr(d1, G, nfield, d, MIX_W, p)[0];
        dK[d] = d1ptr(d1, G, nfield, d, fK, p)[0];
    }
    // M_i (constraints.py:61-97)
    double M[3];
#pragma unroll 1
    for (int i = 0; i < 3; ++i) {
        double first = 0.0, second = 0.0, third = 0.0;
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            first += d1ptr(d1, G, nfield, j, fB + 3 * i + j, p)[0];
            third += der[(6 + 3 * i + j) * cs + p] * dW[j];
        }
#pragma unroll
        for (int s = 0; s < 6; ++s) {
            const double w = (s == 0 || s == 3 || s == 5) ? 1.0 : 2.0;
            second += w * gi[s] * d1ptr(d1, G, nfield, i, fA + s, p)[0];
        }
        M[i] = first - 0.5 * second - 3.0 * third / Wf - (2.0 / 3.0) * dK[i];
    }
    // d_l M_i (constraints.py:186-213), dM[i][l]
    double hW[6];
    hessian(u, d1, G, nfield, CW, MIX_W, c, hW);
    double dM[3][3];
#pragma unroll 1
    for (int i = 0; i < 3; ++i) {
#pragma unroll 1
        for (int l = 0; l < 3; ++l) {
            double divd = 0.0, conf = 0.0, met = 0.0, met2 = 0.0;
#pragma unroll 1
            for (int j = 0; j < 3; ++j) {
                // d_l d_j B_ij
                const int fb = fB + 3 * i + j;
                divd += (l == j) ? D2(der + (6 + 3 * i + j) * cs + p, G, l, c.ix[l])
                                 : mixed(d1, G, nfield, fb, l, j, c);
                const double dBW = D1(der + (15 + 3 * i + j) * cs + p, G, l, c.ix[l]);
                conf += dBW * dW[j] + der[(15 + 3 * i + j) * cs + p] * hW[sym(l, j)];
            }
#pragma unroll 1
            for (int s = 0; s < 6; ++s) {
                const double w = (s == 0 || s == 3 || s == 5) ? 1.0 : 2.0;
                const double dgi = D1(der + s * cs + p, G, l, c.ix[l]);
                met += w * dgi * d1ptr(d1, G, nfield, i, fA + s, p)[0];
                const double d2A = (l == i) ? D2(u + (AXX + s) * cs + p, G, l, c.ix[l])
                                            : mixed(d1, G, nfield, fA + s, l, i, c);
                met2 += w * gi[s] * d2A;
            }
            const double d2K = (l == i) ? D2(u + CK * cs + p, G, l, c.ix[l]) : mixed(d1, G, nfield, fK, l, i, c);
            dM[i][l] = divd - 0.5 * met - 0.5 * met2 - 3.0 * conf - (2.0 / 3.0) * d2K;
        }
    }
    // Christoffels for D_j M_i = d_j M_i - Gamma^k_ij M_k
    double g[6], gl[6];
    load_sym(u, GXX, G, p, g);
    inverse_metric(g, gl);
    double c1[3][6], c2[3][6];
    {
        double dg[3][6];
        load_metric_derivs(d1, G, nfield, p, dg);
        christoffel(dg, gl, c1, c2);
    }
    const double scale = G.kappa / 2.0 * u[CALPHA * cs + p];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = i; j < 3; ++j) {
            const int s = sym(i, j);
            const double gm = c2[0][s] * M[0] + c2[1][s] * M[1] + c2[2][s] * M[2];
            const double DjMi = dM[i][j] - gm;
            const double DiMj = dM[j][i] - gm;
            damp[s * cs + p] = scale * (DjMi + DiMj);
        }
}

// ---------------------------------------------------------------------------
// Sommerfeld faces: rhs = -(x^i/r d_i u + (u - u_inf)/r) (boundaries.py:74-147)
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kThreads)
k_sommerfeld(const double* __restrict__ u, double* __restrict__ k, Geo G, Box B) {
    PointCtx c;
    if (!point(B, c, G)) return;
    bool face = false;
    bool owned = true;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        const Axis& a = G.ax[d];
        owned = owned && c.ix[d] >= a.start && c.ix[d] < a.end;
        face = face || (a.slo && c.ix[d] == a.start) || (a.shi && c.ix[d] == a.end - 1);
    }
    if (!(face && owned)) return;
    double X[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) X[d] = __dadd_rn(G.ax[d].xmin, __dmul_rn(G.dx, (double)(c.ix[d] - G.ax[d].org)));
    const double r = __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(X[0], X[0]), __dmul_rn(X[1], X[1])),
                                          __dmul_rn(X[2], X[2])));
    const double rs = r > 0.0 ? r : 1.0;
    const long long cs = G.cs, p = c.p;
#pragma unroll 1
    for (int comp = 0; comp < NCOMP; ++comp) {
        const double* f = u + comp * cs + p;
        const double radial = (X[0] * D1(f, G, 0, c.ix[0]) + X[1] * D1(f, G, 1, c.ix[1])
                               + X[2] * D1(f, G, 2, c.ix[2])) / rs;
        double asym = 0.0;
        if (comp == GXX || comp == GYY || comp == GZZ || comp == CW || comp == CALPHA) asym = 1.0;
        k[comp * cs + p] = -(radial + (f[0] - asym) / rs);
    }
}

// ---------------------------------------------------------------------------
// Constraint fields (JAX_BSSN/bssn/constraints.py:22-97, 271-412): H, M_i,
// det(gt) - 1, gt^ij At_ij and Gt^i - gt^jk Gamma^i_jk, written in the
// reference layout at the box's linear index.
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
    load_sym(u, GXX, G, p, g);
    load_sym(u, AXX, G, p, A);
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
        dK[d] = D1(u + CK * cs + p, G, d, c.ix[d]);
    }
    const double W = u[CW * cs + p];
    const double K = u[CK * cs + p];
    double w2r[6];
    w2_ricci(u, d1, G, NMIX, c, g, gi, c1, c2, dW, W, w2r);
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
            first += D1(der + (6 + 3 * i + j) * cs + p, G, j, c.ix[j]);
            third += der[(6 + 3 * i + j) * cs + p] * dW[j];
        }
#pragma unroll 1
        for (int s = 0; s < 6; ++s) {
            const double w = (s == 0 || s == 3 || s == 5) ? 1.0 : 2.0;
            second += w * gi[s] * D1(u + (AXX + s) * cs + p, G, i, c.ix[i]);
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
        int lo = box.lo[d] - by, hi = box.lo[d] + box.n[d] + by;
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

cudaError_t launch_constraints(const double* u, const RhsWork& w, const Geo& G, const Box& box, double* H,
                               double* M, double* detm1, double* trA, double* gam, cudaStream_t stream) {
    const Box ext = grown_box(box, G, composition_reach(G));
    // derived fields are pointwise and read on the box only
    BSSN_LAUNCH(KC_MOM_DERIVED, k_mom_derived, blocks_for(ext.count), kThreads, stream, u, w.der, G, ext);
    BSSN_LAUNCH(KC_FIRST, k_first_derivs, blocks_for(ext.count), kThreads, stream, u, w.der, w.d1, G, ext, 0);
    BSSN_LAUNCH(KC_CONSTRAINTS, k_constraints, blocks_for(box.count), kThreads, stream, u, w.d1, w.der, G, box,
                H, M, detm1, trA, gam);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// host-side launch sequence of one RHS evaluation
// ---------------------------------------------------------------------------

cudaError_t launch_rhs(const double* u, double* k, const RhsWork& w, const Geo& G, const Box& box,
                       cudaStream_t stream) {
    const int with_mom = G.kappa != 0.0;
    const int nfield = with_mom ? NMIX + NMIX_MOM : NMIX;
    const int reach = composition_reach(G);
    const Box ext = grown_box(box, G, reach);
    if (with_mom) {
        // The derived fields are differentiated on ext, so they must be valid
        // on ext grown by the first-derivative reach (3); being pointwise, they
        // take the same values there whatever region is computed.
        const Box region = grown_box(box, G, reach + 3);
        BSSN_LAUNCH(KC_MOM_DERIVED, k_mom_derived, blocks_for(region.count), kThreads, stream, u, w.der, G, region);
    }
    BSSN_LAUNCH(KC_FIRST, k_first_derivs, blocks_for(ext.count), kThreads, stream, u, w.der, w.d1, G, ext, with_mom);
    if (with_mom)
        BSSN_LAUNCH(KC_MOM_DAMP, k_mom_damping, blocks_for(box.count), kThreads, stream, u, w.der, w.d1, w.damp, G, box, nfield);
    BSSN_LAUNCH(KC_GAUGE, k_rhs_gauge, blocks_for(box.count), kThreads, stream, u, w.d1, k, G, box, nfield);
    BSSN_LAUNCH(KC_KGT, k_rhs_kgt, blocks_for(box.count), kThreads, stream, u, w.d1, k, G, box, nfield);
    BSSN_LAUNCH(KC_AT, k_rhs_at, blocks_for(box.count), kThreads, stream, u, w.d1, with_mom ? w.damp : nullptr, k, G, box,
                nfield);
    if (G.any_sommerfeld) BSSN_LAUNCH(KC_SOMMERFELD, k_sommerfeld, blocks_for(box.count), kThreads, stream, u, k, G, box);
    return cudaGetLastError();
}

}  // namespace bssn
