// Per-pair quadrature of the four local blocks and their scatter into the CSR accumulators.
//
//   termLocal[a][b]       -> A[aV[a], aV[b]]   (+), row kept if label(aV[a]) > 0
//   termNonloc[a][b]      -> A[aV[a], bV[b]]   (-)
//   termLocalPrime[a][b]  -> A[bV[b], bV[a]]   (+), row kept if label(bV[b]) > 0
//   termNonlocPrime[a][b] -> A[bV[b], aV[a]]   (-)
// (src/Cassemble.cpp:721-770, outdim = 1, no domain-decomposition weight).
#pragma once
#include "geometry.cuh"
#include "primitives.cuh"

namespace nlg {

constexpr int MAXQ = 32;   // points per outer/inner rule

// Quadrature rule on the reference element; passed by value (kernel parameter space).
struct Rule {
    int nPx, nPy, dim, pad;
    double Px[MAXQ * 3], dx[MAXQ], Py[MAXQ * 3], dy[MAXQ];
    double psix[MAXQ * 4], psiy[MAXQ * 4];   // [k * dV + a]
    float Pyf[MAXQ * 2], dyf[MAXQ], psiyf[MAXQ * 4];
    float Pxf[MAXQ * 3];
};

// Duffy tables of the singular close-pair rule (MeshTypes.cpp:252-327), device pointers.
struct Duffy {
    int nPg;
    const double *alpha[3];   // [case][(t * nPg + k) * 4 + j], xi factored out (canceled)
    const double *tdet[3];    // [case][t * nPg + k], xi^(3 - 2s) (fractional rule)
    const double *alphaU[3];  // the points with xi kept (weakSingular basis functions)
    const double *tdetW[3];   // xi^(1 - 2s) (weakSingular)
    const double *dg;         // [k]
    const float4 *alf[3];     // FP32 copies of alpha (mixed path)
    const float *wf[3];       // FP32 tdet * dg (mixed path)
    const float4 *alfU[3];    // FP32 copies of alphaU (mixed weakSingular rule)
    const float *wfW[3];      // FP32 tdetW * dg (mixed weakSingular rule)
};

struct QuadArgs {
    const int *pA, *pB, *T32, *labV, *eprob;
    const int *labT;          // element labels (label-dependent kernels)
    const double *EC, *adet;
    const ProbParams *probs;
    const long long *rowptr;
    const int *cols;
    unsigned long long *acc;
    unsigned *tiny;
    long long P;
    const int *list;          // optional index list into the pairs
    long long nlist;
    int *err;                 // [3] slot not found, [4] singular toRef, [7] kernel outside its domain
    unsigned long long *n_close;
    double *blocks_out;       // explicit-pair mode: (P, 4, dV, dV) blocks instead of scatter
    int *ret_out;             // explicit-pair mode: doesInteract
    int force_close;          // explicit-pair mode: use the close-pair rule
    unsigned long long *n_subtri;
};

__device__ __forceinline__ long long find_slot(const long long *__restrict__ rowptr,
                                               const int *__restrict__ cols, int row, int col) {
    long long lo = rowptr[row], hi = rowptr[row + 1] - 1;
    while (lo <= hi) {
        long long mid = (lo + hi) >> 1;
        int c = cols[mid];
        if (c == col) return mid;
        if (c < col) lo = mid + 1; else hi = mid - 1;
    }
    return -1;
}

__device__ __forceinline__ void add_entry(const QuadArgs &a, int row, int col, double val, int se) {
    long long s = find_slot(a.rowptr, a.cols, row, col);
    if (s < 0) { atomicOr(&a.err[3], 1); return; }
    fx_atomic_add(&a.acc[2 * s], val, se, &a.tiny[s]);
}

template <int dV>
__device__ __forceinline__ void scatter_blocks(const QuadArgs &a, const int *aV, const int *bV,
                                               const double *L, const double *N, const double *LP,
                                               const double *NP, int se, bool prime) {
#pragma unroll 1
    for (int i = 0; i < dV; i++) {
        if (a.labV[aV[i]] > 0) {
            for (int j = 0; j < dV; j++) {
                add_entry(a, aV[i], aV[j], L[dV * i + j], se);
                add_entry(a, aV[i], bV[j], -N[dV * i + j], se);
            }
        }
    }
    if (!prime) return;
#pragma unroll 1
    for (int j = 0; j < dV; j++) {
        if (a.labV[bV[j]] > 0) {
            for (int i = 0; i < dV; i++) {
                add_entry(a, bV[j], bV[i], LP[dV * i + j], se);
                add_entry(a, bV[j], aV[i], -NP[dV * i + j], se);
            }
        }
    }
}

__device__ __forceinline__ bool share_vertex(const int *aV, const int *bV, int dV) {
    for (int i = 0; i < dV; i++)
        for (int j = 0; j < dV; j++)
            if (aV[i] == bV[j]) return true;
    return false;
}

// FP64 integrate_retriangulate (integration.cpp:345-540) of one pair.
__device__ int quad_retriangulate_f64(const ProbParams &P, const Rule &rule, const double *Ea,
                                      const double *Eb, int la, int lb, double adet_a, double *L, double *N,
                                      double *LP, double *NP, int *err, int &nsub) {
    double R[18];
    int interacts = 0;
    for (int k = 0; k < rule.nPx; k++) {
        double x[2];
        xtoPhys<2>(Ea, &rule.Px[2 * k], x);
        const int Rdx = xretriangulate(x, Eb, P.sqdelta, P.caps, R);
        interacts |= (Rdx >= 3);
        nsub += Rdx >= 3 ? Rdx - 2 : 0;
        double innerLocal = 0, iN[3] = {0, 0, 0}, iNP[3] = {0, 0, 0};
        for (int r = 0; r + 2 < Rdx; r++) {
            const double tri[6] = {R[0], R[1], R[2 * r + 2], R[2 * r + 3], R[2 * r + 4], R[2 * r + 5]};
            const double rTdet = xabsDet2(tri);
            for (int i = 0; i < rule.nPy; i++) {
                double y[2];
                // toPhys(E, p, out) of the sub-triangle (mathhelpers.cpp:210-215)
                y[0] = (tri[2] - tri[0]) * rule.Py[2 * i] + (tri[4] - tri[0]) * rule.Py[2 * i + 1] + tri[0];
                y[1] = (tri[3] - tri[1]) * rule.Py[2 * i] + (tri[5] - tri[1]) * rule.Py[2 * i + 1] + tri[1];
                const double ker = kernel_f64<2>(P, x, la, y, lb, err);
                const double w = rule.dy[i] * rTdet;
                innerLocal += ker * w;
                double ref[2];
                if (!xtoRef(Eb, y, ref)) atomicOr(&err[4], 1);
                const double kerP = kernel_f64<2>(P, y, lb, x, la, err);
                const double psi[3] = {1.0 - ref[0] - ref[1], ref[0], ref[1]};
                const double wl = kerP * w * rule.dx[k] * adet_a;
#pragma unroll
                for (int b = 0; b < 3; b++) {
                    iN[b] += psi[b] * ker * w;
                    iNP[b] += psi[b] * kerP * w;
                }
#pragma unroll
                for (int aa = 0; aa < 3; aa++)
#pragma unroll
                    for (int b = 0; b < 3; b++) LP[3 * aa + b] += psi[aa] * psi[b] * wl;
            }
        }
        const double wx = adet_a * rule.dx[k];
#pragma unroll
        for (int aa = 0; aa < 3; aa++) {
            const double pa = rule.psix[3 * k + aa] * wx;
#pragma unroll
            for (int b = 0; b < 3; b++) {
                L[3 * aa + b] += pa * rule.psix[3 * k + b] * innerLocal;
                N[3 * aa + b] += pa * iN[b];
                NP[3 * aa + b] += pa * iNP[b];
            }
        }
    }
    return interacts | P.full_search;
}

// FP64 integrate_baryCenter (integration.cpp:910-1018) of one pair (2D or 3D).
template <int DIM>
__device__ int quad_barycenter_f64(const ProbParams &P, const Rule &rule, const double *Ea,
                                   const double *Eb, int la, int lb, double adet_a, double adet_b, double *L,
                                   double *N, int *err, int &nsub) {
    constexpr int dV = DIM + 1;
    double b[DIM];
    xbary<DIM>(Eb, b);
    int interacts = 0;
    for (int k = 0; k < rule.nPx; k++) {
        double x[DIM];
        xtoPhys<DIM>(Ea, &rule.Px[DIM * k], x);
        if (!xbaryInside<DIM>(x, b, P.sqdelta)) continue;
        interacts = 1;
        nsub++;
        double innerLocal = 0, iN[dV];
#pragma unroll
        for (int j = 0; j < dV; j++) iN[j] = 0;
        for (int i = 0; i < rule.nPy; i++) {
            double y[DIM];
            xtoPhys<DIM>(Eb, &rule.Py[DIM * i], y);
            const double ker = kernel_f64<DIM>(P, x, la, y, lb, err);
            innerLocal += adet_b * ker * rule.dy[i];
            const double kerP = kernel_f64<DIM>(P, y, lb, x, la, err);
#pragma unroll
            for (int j = 0; j < dV; j++) iN[j] += rule.psiy[dV * i + j] * kerP * rule.dy[i] * adet_b;
        }
        const double wx = 2.0 * adet_a * rule.dx[k];
#pragma unroll
        for (int aa = 0; aa < dV; aa++) {
            const double pa = rule.psix[dV * k + aa] * wx;
#pragma unroll
            for (int j = 0; j < dV; j++) {
                L[dV * aa + j] += pa * rule.psix[dV * k + j] * innerLocal;
                N[dV * aa + j] += pa * iN[j];
            }
        }
    }
    return interacts | P.full_search;
}

// ---------------------------------------------------------------- further FP64 rules (2D)
// Out side of the pair (aT, bT) for the rules retriangulate_unsymm, subSetBall / averageBall,
// baryCenterRT and noTruncation. L is the upper triangle of termLocal, N[a][b] termNonloc (a: aT's
// vertex, b: bT's vertex). Except for baryCenterRT, the blocks leave out the factor |aT|, which
// the caller applies. Returns doesInteract without is_fullConnectedComponentSearch.

// integrate_retriangulate_unysmm (integration.cpp:542-704): the retriangulated inner domain, weight
// 2; termNonloc takes k(y, x).
__device__ int rule_retri_unsymm(const ProbParams &P, const Rule &rule, const double *Ea, const double *Eb,
                                 int la, int lb, double *L, double *N, unsigned &nsub, int *err) {
    double R[18];
    int hit = 0;
    for (int k = 0; k < rule.nPx; k++) {
        double x[2];
        xtoPhys<2>(Ea, &rule.Px[2 * k], x);
        const int Rdx = xretriangulate(x, Eb, P.sqdelta, P.caps, R);
        hit |= Rdx >= 3;
        double iL = 0, iN[3] = {0, 0, 0};
        for (int r = 0; r + 2 < Rdx; r++) {
            nsub++;
            const double tri[6] = {R[0], R[1], R[2 * r + 2], R[2 * r + 3], R[2 * r + 4], R[2 * r + 5]};
            const double rTdet = xabsDet2(tri);
            for (int i = 0; i < rule.nPy; i++) {
                double y[2];
                y[0] = (tri[2] - tri[0]) * rule.Py[2 * i] + (tri[4] - tri[0]) * rule.Py[2 * i + 1] + tri[0];
                y[1] = (tri[3] - tri[1]) * rule.Py[2 * i] + (tri[5] - tri[1]) * rule.Py[2 * i + 1] + tri[1];
                const double w = rule.dy[i] * rTdet;
                iL += kernel_f64<2>(P, x, la, y, lb, err) * w;
                double ref[2];
                if (!xtoRef(Eb, y, ref)) atomicOr(&err[4], 1);
                const double kp = kernel_f64<2>(P, y, lb, x, la, err) * w;
                iN[0] += (1.0 - ref[0] - ref[1]) * kp;
                iN[1] += ref[0] * kp;
                iN[2] += ref[1] * kp;
            }
        }
        for (int a = 0; a < 3; a++) {
            const double pa = 2.0 * rule.psix[3 * k + a] * rule.dx[k];
            for (int b = a; b < 3; b++) L[sym_idx<3>(a, b)] += pa * rule.psix[3 * k + b] * iL;
            for (int b = 0; b < 3; b++) N[3 * a + b] += pa * iN[b];
        }
    }
    return hit;
}

// integrate_subSuperSetBalls (integration.cpp:1021-1095) with method_subSuperSetBalls
// (:1251-1260): the whole inner element, weighted by the number n of its vertices strictly inside
// the ball (subSetBall: 1 for n = 3, else 0; averageBall: 1 for n = 3, else 0.5), weight 2.
__device__ int rule_subset(const ProbParams &P, const Rule &rule, const double *Ea, const double *Eb,
                           double adetb, int la, int lb, double *L, double *N, unsigned &nsub, int *err) {
    const double wpart = P.remote == MTH_AVERAGE ? 0.5 : 0.0;
    int hit = 0;
    for (int k = 0; k < rule.nPx; k++) {
        double x[2];
        xtoPhys<2>(Ea, &rule.Px[2 * k], x);
        int n = 0;
        for (int v = 0; v < 3; v++) n += xsqdist2(&Eb[2 * v], x) < P.sqdelta;
        if (n == 0) continue;   // the reference adds zeros
        hit = 1;
        nsub++;
        const double w = n == 3 ? 1.0 : wpart;
        double iL = 0, iN[3] = {0, 0, 0};
        for (int i = 0; i < rule.nPy; i++) {
            double y[2];
            xtoPhys<2>(Eb, &rule.Py[2 * i], y);
            iL += w * adetb * kernel_f64<2>(P, x, la, y, lb, err) * rule.dy[i];
            const double kp = kernel_f64<2>(P, y, lb, x, la, err);
            for (int b = 0; b < 3; b++) iN[b] += w * rule.psiy[3 * i + b] * kp * rule.dy[i] * adetb;
        }
        for (int a = 0; a < 3; a++) {
            const double pa = 2.0 * rule.psix[3 * k + a] * rule.dx[k];
            for (int b = a; b < 3; b++) L[sym_idx<3>(a, b)] += pa * rule.psix[3 * k + b] * iL;
            for (int b = 0; b < 3; b++) N[3 * a + b] += pa * iN[b];
        }
    }
    return hit;
}

// integrate_baryCenterRT (integration.cpp:1155-1249): the outer domain is the part of aT inside the
// ball around bT's barycenter (retriangulated), the inner element is whole, weight 2; the blocks
// carry their factor 2 |sub-triangle|. The reference reads innerNonloc[outdim (a % outdim) +
// b % outdim], which is innerNonloc[0] (the first basis function) for every b at outdim 1.
__device__ int rule_baryrt(const ProbParams &P, const Rule &rule, const double *Ea, const double *Eb,
                           double adetb, int la, int lb, double *L, double *N, unsigned &nsub, int *err) {
    double bc[2];
    xbary<2>(Eb, bc);
    double R[18];
    const int Rdx = xretriangulate(bc, Ea, P.sqdelta, P.caps, R);
    for (int r = 0; r + 2 < Rdx; r++) {
        nsub++;
        const double tri[6] = {R[0], R[1], R[2 * r + 2], R[2 * r + 3], R[2 * r + 4], R[2 * r + 5]};
        const double rTdet = xabsDet2(tri);
        for (int k = 0; k < rule.nPx; k++) {
            double xq[2];
            xtoPhys<2>(tri, &rule.Px[2 * k], xq);
            double iL = 0, iN0 = 0;
            for (int i = 0; i < rule.nPy; i++) {
                double y[2];
                xtoPhys<2>(Eb, &rule.Py[2 * i], y);
                iL += kernel_f64<2>(P, xq, la, y, lb, err) * rule.dy[i] * adetb;
                iN0 += rule.psiy[3 * i] * kernel_f64<2>(P, y, lb, xq, la, err) * rule.dy[i] * adetb;
            }
            double ref[2];
            if (!xtoRef(Ea, xq, ref)) atomicOr(&err[4], 1);
            const double ps[3] = {1.0 - ref[0] - ref[1], ref[0], ref[1]};
            for (int a = 0; a < 3; a++) {
                const double pa = 2.0 * rTdet * ps[a];
                for (int b = a; b < 3; b++) L[sym_idx<3>(a, b)] += pa * ps[b] * rule.dx[k] * iL;
                for (int b = 0; b < 3; b++) N[3 * a + b] += pa * rule.dx[k] * iN0;
            }
        }
    }
    return Rdx >= 3;
}

// integrate_fullyContained (integration.cpp:290-343), "noTruncation": both elements whole, every
// pair interacts. Out side of (aT, bT): termLocal with k(x, y), termNonloc with k(y, x).
__device__ void rule_notrunc_out(const ProbParams &P, const Rule &rule, const double *Ea, const double *Eb,
                                 double adetb, int la, int lb, double *L, double *N, int *err) {
    for (int k = 0; k < rule.nPx; k++) {
        double x[2];
        xtoPhys<2>(Ea, &rule.Px[2 * k], x);
        for (int i = 0; i < rule.nPy; i++) {
            double y[2];
            xtoPhys<2>(Eb, &rule.Py[2 * i], y);
            const double kv = kernel_f64<2>(P, x, la, y, lb, err);
            const double kp = kernel_f64<2>(P, y, lb, x, la, err);
            const double f = rule.dx[k] * rule.dy[i] * adetb;
            for (int a = 0; a < 3; a++) {
                const double fa = f * rule.psix[3 * k + a];
                for (int b = a; b < 3; b++) L[sym_idx<3>(a, b)] += fa * rule.psix[3 * k + b] * kv;
                for (int b = 0; b < 3; b++) N[3 * a + b] += fa * rule.psiy[3 * i + b] * kp;
            }
        }
    }
}
// Prime side of (aT, bT): termLocalPrime (upper triangle, bT's vertices) with k(y, x) and
// termNonlocPrime[a][b] (a: aT's vertex, b: bT's vertex) with k(x, y), without |aT|.
__device__ __noinline__ void rule_notrunc_prime(const ProbParams &P, const Rule &rule, const double *Ea, const double *Eb,
                                   double adetb, int la, int lb, double *LP, double *NP, int *err) {
    for (int k = 0; k < rule.nPx; k++) {
        double x[2];
        xtoPhys<2>(Ea, &rule.Px[2 * k], x);
        for (int i = 0; i < rule.nPy; i++) {
            double y[2];
            xtoPhys<2>(Eb, &rule.Py[2 * i], y);
            const double kv = kernel_f64<2>(P, x, la, y, lb, err);
            const double kp = kernel_f64<2>(P, y, lb, x, la, err);
            const double f = rule.dx[k] * rule.dy[i] * adetb;
            for (int a = 0; a < 3; a++) {
                const double fa = f * rule.psiy[3 * i + a];
                for (int b = a; b < 3; b++) LP[sym_idx<3>(a, b)] += fa * rule.psiy[3 * i + b] * kp;
                const double fx = f * rule.psix[3 * k + a];
                for (int b = 0; b < 3; b++) NP[3 * a + b] += fx * rule.psiy[3 * i + b] * kv;
            }
        }
    }
}

// integrate_exact, "exactBall" (integration.cpp:706-907): per outer point the polygon of
// method_exact (fan sub-triangles, the inner rule on each) plus its circular segments, each at its
// centroid with its area as weight; weight 2, no prime blocks. The blocks leave out |aT|.
__device__ int rule_exact(const ProbParams &P, const Rule &rule, const double *Ea, const double *Eb,
                          int la, int lb, double *L, double *N, unsigned &nsub, int *err) {
    int interacts = 0;
    for (int k = 0; k < rule.nPx; k++) {
        double x[2], R[18], caps[6], capw[3];
        int ncaps = 0;
        xtoPhys<2>(Ea, &rule.Px[2 * k], x);
        const int n = xmethod_exact(x, Eb, P.sqdelta, R, caps, capw, &ncaps);
        interacts |= n >= 3;
        double iL = 0, iN[3] = {0, 0, 0};
        for (int r = 0; r + 2 < n; r++) {
            nsub++;
            const double tri[6] = {R[0], R[1], R[2 * r + 2], R[2 * r + 3], R[2 * r + 4], R[2 * r + 5]};
            const double rTdet = xabsDet2(tri);
            for (int i = 0; i < rule.nPy; i++) {
                double y[2];
                y[0] = (tri[2] - tri[0]) * rule.Py[2 * i] + (tri[4] - tri[0]) * rule.Py[2 * i + 1] + tri[0];
                y[1] = (tri[3] - tri[1]) * rule.Py[2 * i] + (tri[5] - tri[1]) * rule.Py[2 * i + 1] + tri[1];
                iL += kernel_f64<2>(P, x, la, y, lb, err) * rule.dy[i] * rTdet;
                double ref[2];
                if (!xtoRef(Eb, y, ref)) atomicOr(&err[4], 1);
                const double kp = kernel_f64<2>(P, y, lb, x, la, err);
                const double psi[3] = {1.0 - ref[0] - ref[1], ref[0], ref[1]};
                for (int b = 0; b < 3; b++) iN[b] += psi[b] * kp * rule.dy[i] * rTdet;
            }
        }
        for (int c = 0; c < ncaps; c++) {
            iL += kernel_f64<2>(P, x, la, &caps[2 * c], lb, err) * capw[c];
            double ref[2];
            if (!xtoRef(Eb, &caps[2 * c], ref)) atomicOr(&err[4], 1);
            const double kp = kernel_f64<2>(P, &caps[2 * c], lb, x, la, err);
            const double psi[3] = {1.0 - ref[0] - ref[1], ref[0], ref[1]};
            for (int b = 0; b < 3; b++) iN[b] += psi[b] * kp * capw[c];
        }
        for (int a = 0; a < 3; a++) {
            const double pa = 2.0 * rule.psix[3 * k + a];
            for (int b = a; b < 3; b++) L[sym_idx<3>(a, b)] += pa * rule.psix[3 * k + b] * rule.dx[k] * iL;
            for (int b = 0; b < 3; b++) N[3 * a + b] += pa * rule.dx[k] * iN[b];
        }
    }
    return interacts;
}

// Out of line: the rules are rare, and inlined they would take registers from the passes' common
// paths.
__device__ __noinline__ int rule_out_f64(const ProbParams &P, int method, const Rule &rule, const double *Ea, const double *Eb,
                            double adetb, int la, int lb, double *L, double *N, unsigned &nsub, int *err) {
    switch (method) {
    case MTH_RETRI_UNSYMM: return rule_retri_unsymm(P, rule, Ea, Eb, la, lb, L, N, nsub, err);
    case MTH_SUBSET: case MTH_AVERAGE: return rule_subset(P, rule, Ea, Eb, adetb, la, lb, L, N, nsub, err);
    case MTH_BARY_RT: return rule_baryrt(P, rule, Ea, Eb, adetb, la, lb, L, N, nsub, err);
    case MTH_NOTRUNC: nsub += rule.nPx; rule_notrunc_out(P, rule, Ea, Eb, adetb, la, lb, L, N, err); return 1;
    case MTH_EXACT: return rule_exact(P, rule, Ea, Eb, la, lb, L, N, nsub, err);
    }
    return 0;
}

// One thread per (non-close) pair: FP64 quadrature and scatter.
template <int DIM>
__global__ void __launch_bounds__(128) k_quad_fp64(QuadArgs a, Rule rule) {
    constexpr int dV = DIM + 1;
    const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    int nsub = 0;
    if (p < a.P) {
        const int aT = a.pA[p], bT = a.pB[p];
        const ProbParams P = a.probs[a.eprob[aT]];
        int aV[dV], bV[dV];
#pragma unroll
        for (int i = 0; i < dV; i++) { aV[i] = a.T32[(long long)aT * dV + i]; bV[i] = a.T32[(long long)bT * dV + i]; }
        const bool close = a.blocks_out ? (a.force_close != 0) : (P.singular && share_vertex(aV, bV, dV));
        const int method = close ? P.close : P.remote;
        if (method != MTH_FRACTIONAL && method != MTH_WEAKSING) {   // Duffy close pairs: k_quad_close
            double Ea[DIM * dV], Eb[DIM * dV];
#pragma unroll
            for (int i = 0; i < DIM * dV; i++) { Ea[i] = a.EC[(long long)aT * DIM * dV + i]; Eb[i] = a.EC[(long long)bT * DIM * dV + i]; }
            double L[dV * dV], N[dV * dV], LP[dV * dV], NP[dV * dV];
#pragma unroll
            for (int i = 0; i < dV * dV; i++) { L[i] = 0; N[i] = 0; LP[i] = 0; NP[i] = 0; }
            bool prime = false;
            int interacts = 0;
            if (method == MTH_BARYCENTER) {
                interacts = quad_barycenter_f64<DIM>(P, rule, Ea, Eb, a.labT[aT], a.labT[bT], a.adet[aT], a.adet[bT], L, N, a.err, nsub);
            } else if (DIM == 2 && method == MTH_RETRIANGULATE) {
                interacts = quad_retriangulate_f64(P, rule, Ea, Eb, a.labT[aT], a.labT[bT], a.adet[aT], L, N, LP, NP, a.err, nsub);
                prime = true;
            } else if (DIM == 2) {
                double Ls[6] = {0, 0, 0, 0, 0, 0}, LPs[6] = {0, 0, 0, 0, 0, 0};
                unsigned ns = 0;
                interacts = rule_out_f64(P, method, rule, Ea, Eb, a.adet[bT], a.labT[aT], a.labT[bT], Ls, N, ns, a.err) | P.full_search;
                if (method == MTH_NOTRUNC) {
                    rule_notrunc_prime(P, rule, Ea, Eb, a.adet[bT], a.labT[aT], a.labT[bT], LPs, NP, a.err);
                    prime = true;
                }
                const double sa = method == MTH_BARY_RT ? 1.0 : a.adet[aT];
                for (int i = 0; i < 3; i++)
                    for (int j = 0; j < 3; j++) {
                        const int sij = i <= j ? sym_idx<3>(i, j) : sym_idx<3>(j, i);
                        L[3 * i + j] = Ls[sij] * sa;
                        LP[3 * i + j] = LPs[sij] * sa;
                    }
                for (int i = 0; i < 9; i++) { N[i] *= sa; NP[i] *= sa; }
                nsub += (int)ns;
            }
            if (a.blocks_out) {
                double *o = &a.blocks_out[p * 4 * dV * dV];
                for (int i = 0; i < dV * dV; i++) {
                    o[i] = L[i]; o[dV * dV + i] = N[i]; o[2 * dV * dV + i] = LP[i]; o[3 * dV * dV + i] = NP[i];
                }
                a.ret_out[p] = interacts;
            } else {
                scatter_blocks<dV>(a, aV, bV, L, N, LP, NP, P.scale_exp, prime);
            }
        }
    }
    const unsigned tot = __reduce_add_sync(FULL, (unsigned)nsub);
    if ((threadIdx.x & 31) == 0 && tot && a.n_subtri) atomicAdd(a.n_subtri, (unsigned long long)tot);
}

// Flags and lists the close pairs (singular kernel, shared vertex, Duffy close rule).
template <int DIM>
__global__ void k_close_list(QuadArgs a, int *list, unsigned long long *count) {
    constexpr int dV = DIM + 1;
    const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= a.P) return;
    const int aT = a.pA[p], bT = a.pB[p];
    const ProbParams &P = a.probs[a.eprob[aT]];
    if (!duffy_close(P)) return;
    int aV[dV], bV[dV];
    for (int i = 0; i < dV; i++) { aV[i] = a.T32[(long long)aT * dV + i]; bV[i] = a.T32[(long long)bT * dV + i]; }
    if (!share_vertex(aV, bV, dV)) return;
    unsigned long long i = atomicAdd(count, 1ULL);
    list[i] = (int)p;
}

// One warp per close pair: integrate_fractional (integration.cpp:187-288) with join()
// (:1913-1958), FP64 throughout; lanes stride over the Duffy points, warp-reduce the blocks.
// r2^h (h < 0) for the mixed path: r2 = m 2^E exactly (frexp, m in [1/2, 1)), and h E = I + f
// with I = floor(h E) an integer, so r2^h = 2^I 2^(f + h log2 m) where only the last power, of an
// argument in [0, 1 - h), is evaluated in FP32 (exp2f, log2f). Its relative error is a few units
// of 2^-24 times (1 + |h|), about 3e-7, far inside the mixed path's 1e-6; the binary exponent
// is exact. Range reduction by the exact power of two, as in any pow implementation.
__device__ __forceinline__ double pow_split(double r2, double h) {
    int E;
    const double m = frexp(r2, &E);
    const double t = h * (double)E;
    const double I = floor(t);
    const float g = fmaf((float)h, log2f((float)m), (float)(t - I));
    return ldexp((double)exp2f(g), (int)I);
}

// Sum over the Duffy points of one close pair (integration.cpp:187-288) of w pxy pxy^T, upper
// triangle of the nL x nL matrix, nL = 6 - NEQ: the lanes take the (map, Gauss point) items in
// turn. The kernel value |x - y|^-(d+2s) is taken as exp2(-(d+2s)/2 log2 |x - y|^2), the same
// function as the reference's 1/pow(sqrt(r), d+2s) without the power's extra work; FAST (mixed
// path) evaluates it with pow_split and sums in compensated FP32.
template <int NEQ, bool FAST>
__device__ __forceinline__ void close_accumulate(const ProbParams &P, const Duffy &d, int c, int nT,
                                                 const double *EA, const double *EB, double dAB, double *M) {
    constexpr int NL = 6 - NEQ, SH = 3 - NEQ;
    const int lane = threadIdx.x & 31;
    const int total = nT * d.nPg;
    const double *al_base = d.alpha[c];
    const double *td_base = d.tdet[c];
    const double a0 = EA[2] - EA[0], a1 = EA[4] - EA[0], a2 = EA[3] - EA[1], a3 = EA[5] - EA[1];
    const double b0 = EB[2] - EB[0], b1 = EB[4] - EB[0], b2 = EB[3] - EB[1], b3 = EB[5] - EB[1];
    const double hexp = -0.5 * P.expo;
    float Mf[FAST ? 21 : 1], Mc[FAST ? 21 : 1];   // FAST: FP32 sums and their compensation
#pragma unroll
    for (int q = 0; q < (FAST ? 21 : 1); q++) Mf[q] = Mc[q] = 0.f;
    for (int idx = lane; idx < total; idx += 32) {
        const int k = idx % d.nPg;
        const double *al = &al_base[(long long)idx * 4];
        const double tf = td_base[idx];
        const double x0 = al[0] * a0 + al[1] * a1 + EA[0], x1 = al[0] * a2 + al[1] * a3 + EA[1];
        const double y0 = al[2] * b0 + al[3] * b1 + EB[0], y1 = al[2] * b2 + al[3] * b3 + EB[1];
        const double z0 = x0 - y0, z1 = x1 - y1;
        const double r2 = z0 * z0 + z1 * z1;
        const double ker = P.kc * (FAST ? pow_split(r2, hexp) : exp2(hexp * log2(r2)));
        const double px[3] = {1.0 - al[0] - al[1], al[0], al[1]};
        const double py[3] = {1.0 - al[2] - al[3], al[2], al[3]};
        double v[NL];
#pragma unroll
        for (int i = 0; i < 3; i++) {
            if (i < NEQ) {
                v[i] = px[i] - py[i];
            } else {
                v[i] = px[i];
                v[i + SH] = -py[i];
            }
        }
        const double base = ker * tf * d.dg[k] * dAB;
        if (FAST) {
            // mixed path: the summands, each a product of FP64 values rounded once to FP32, are
            // added with Kahan compensation (error about 2^-23 of the sum, independent of the
            // point count); the lanes' sums are combined in FP64 by the caller
            float vf[NL];
#pragma unroll
            for (int aa = 0; aa < NL; aa++) vf[aa] = (float)v[aa];
            const float bf = (float)base;
#pragma unroll
            for (int aa = 0; aa < NL; aa++) {
                const float fa = bf * vf[aa];
#pragma unroll
                for (int b = aa; b < NL; b++) {
                    const int q = sym_idx<6>(aa, b);
                    const float y = fmaf(fa, vf[b], -Mc[q]);
                    const float t = Mf[q] + y;
                    Mc[q] = (t - Mf[q]) - y;
                    Mf[q] = t;
                }
            }
        } else {
#pragma unroll
            for (int aa = 0; aa < NL; aa++) {
                const double fa = base * v[aa];
#pragma unroll
                for (int b = aa; b < NL; b++) M[sym_idx<6>(aa, b)] += fa * v[b];
            }
        }
    }
    if (FAST) {
#pragma unroll
        for (int q = 0; q < 21; q++) M[q] = (double)Mf[q] - (double)Mc[q];
    }
}

// The same sum on the mixed path with FP32 arithmetic throughout the point loop (FP64 runs at
// 1/64 of the FP32 rate here). The pair's first vertex is shared (the join puts the common vertices
// first), so x - y = al0 a0 + al1 a1 - al2 b0 - al3 b1 with the edge vectors a, b of both elements
// from that vertex; the edge vectors enter as FP32 hi + lo parts, which keeps x - y accurate to a
// few units of 2^-24 of its size (the canceled Duffy maps keep |x - y| of the order of the
// edges). The power r2^h, h = -(d+2s)/2, takes the exact binary exponent of r2 = m 2^E:
// r2^h = 2^I 2^(t - I + h log2 m), t = h E, I = floor(t), with h split into hh (12 significant
// bits, so hh E is exact) and hl, so only arguments in [-2, 2] reach exp2f and log2f. Each
// summand w kc dAB ker pxy pxy^T is added with Kahan compensation; the lanes' sums are combined in
// FP64 by the caller.
template <int NEQ>
__device__ __forceinline__ void close_accumulate_f32(const ProbParams &P, const Duffy &d, int c, int nT,
                                                     const double *EA, const double *EB, double dAB, double *M) {
    constexpr int NL = 6 - NEQ, SH = 3 - NEQ;
    const int lane = threadIdx.x & 31;
    const int total = nT * d.nPg;
    const float4 *alf = d.alf[c];
    const float *wf = d.wf[c];
    const double ae[4] = {EA[2] - EA[0], EA[4] - EA[0], EA[3] - EA[1], EA[5] - EA[1]};
    const double be[4] = {EB[2] - EB[0], EB[4] - EB[0], EB[3] - EB[1], EB[5] - EB[1]};
    float ah[4], al[4], bh[4], bl[4];
#pragma unroll
    for (int i = 0; i < 4; i++) {
        ah[i] = (float)ae[i]; al[i] = (float)(ae[i] - (double)ah[i]);
        bh[i] = (float)be[i]; bl[i] = (float)(be[i] - (double)bh[i]);
    }
    const double hexp = -0.5 * P.expo;
    const float hh = (float)(ldexp(rint(ldexp(hexp, 8)), -8));   // 8 fraction bits, |h| < 16: exact products with E
    const float hl = (float)(hexp - (double)hh);
    const float hf = (float)hexp;
    const float kcd = (float)(P.kc * dAB);
    float Mf[21], Mc[21];
#pragma unroll
    for (int q = 0; q < 21; q++) Mf[q] = Mc[q] = 0.f;
    for (int idx = lane; idx < total; idx += 32) {
        const float4 a4 = alf[idx];
        const float w = wf[idx];
        float z0 = fmaf(a4.x, ah[0], fmaf(a4.y, ah[1], fmaf(-a4.z, bh[0], -a4.w * bh[1])));
        float z1 = fmaf(a4.x, ah[2], fmaf(a4.y, ah[3], fmaf(-a4.z, bh[2], -a4.w * bh[3])));
        z0 = fmaf(a4.x, al[0], fmaf(a4.y, al[1], fmaf(-a4.z, bl[0], fmaf(-a4.w, bl[1], z0))));
        z1 = fmaf(a4.x, al[2], fmaf(a4.y, al[3], fmaf(-a4.z, bl[2], fmaf(-a4.w, bl[3], z1))));
        const float r2 = fmaf(z0, z0, z1 * z1);
        int E;
        const float m = frexpf(r2, &E);
        const float t = hh * (float)E;   // exact
        const float I = floorf(t);
        const float g = fmaf(hf, log2f(m), fmaf(hl, (float)E, t - I));
        const float ker = ldexpf(exp2f(g), (int)I);
        const float px[3] = {1.f - a4.x - a4.y, a4.x, a4.y};
        const float py[3] = {1.f - a4.z - a4.w, a4.z, a4.w};
        float v[NL];
#pragma unroll
        for (int i = 0; i < 3; i++) {
            if (i < NEQ) {
                v[i] = px[i] - py[i];
            } else {
                v[i] = px[i];
                v[i + SH] = -py[i];
            }
        }
        const float bf = ker * w * kcd;
#pragma unroll
        for (int aa = 0; aa < NL; aa++) {
            const float fa = bf * v[aa];
#pragma unroll
            for (int b = aa; b < NL; b++) {
                const int q = sym_idx<6>(aa, b);
                const float y = fmaf(fa, v[b], -Mc[q]);
                const float tt = Mf[q] + y;
                Mc[q] = (tt - Mf[q]) - y;
                Mf[q] = tt;
            }
        }
    }
#pragma unroll
    for (int q = 0; q < 21; q++) M[q] = (double)Mf[q] - (double)Mc[q];
}

// integrate_weakSingular (integration.cpp:82-185), the lanes taking the (map, Gauss point) items
// in turn: the kernel at the canceled points (as in the fractional rule), the basis functions at
// the points with xi kept, the weight xi^(1 - 2s). W holds termLocal and termLocalPrime (upper
// triangles) and termNonloc (3 x 3), all in the order of the join's sorted vertices.
__device__ __forceinline__ void weak_accumulate(const ProbParams &P, const Duffy &d, int c, int nT,
                                                const double *EA, const double *EB, double dAB, double *W) {
    const int lane = threadIdx.x & 31;
    const int total = nT * d.nPg;
    const double a0 = EA[2] - EA[0], a1 = EA[4] - EA[0], a2 = EA[3] - EA[1], a3 = EA[5] - EA[1];
    const double b0 = EB[2] - EB[0], b1 = EB[4] - EB[0], b2 = EB[3] - EB[1], b3 = EB[5] - EB[1];
    const double hexp = -0.5 * P.expo;
    for (int idx = lane; idx < total; idx += 32) {
        const int k = idx % d.nPg;
        const double *ac = &d.alpha[c][(long long)idx * 4];
        const double *au = &d.alphaU[c][(long long)idx * 4];
        const double x0 = ac[0] * a0 + ac[1] * a1 + EA[0], x1 = ac[0] * a2 + ac[1] * a3 + EA[1];
        const double y0 = ac[2] * b0 + ac[3] * b1 + EB[0], y1 = ac[2] * b2 + ac[3] * b3 + EB[1];
        const double z0 = x0 - y0, z1 = x1 - y1;
        const double ker = P.kc * exp2(hexp * log2(z0 * z0 + z1 * z1));
        const double f = ker * d.tdetW[c][idx] * d.dg[k] * dAB;
        const double px[3] = {1.0 - au[0] - au[1], au[0], au[1]};
        const double py[3] = {1.0 - au[2] - au[3], au[2], au[3]};
#pragma unroll
        for (int i = 0; i < 3; i++) {
            const double fx = f * px[i], fy = f * py[i];
#pragma unroll
            for (int j = i; j < 3; j++) {
                W[sym_idx<3>(i, j)] += fx * px[j];
                W[6 + sym_idx<3>(i, j)] += fy * py[j];
            }
#pragma unroll
            for (int j = 0; j < 3; j++) W[12 + 3 * i + j] += fx * py[j];
        }
    }
}

// The weakSingular sums on the mixed path, in FP32 as close_accumulate_f32 (the same x - y and
// power), with the basis functions at the points with xi kept and the weight xi^(1 - 2s).
__device__ __forceinline__ void weak_accumulate_f32(const ProbParams &P, const Duffy &d, int c, int nT,
                                                    const double *EA, const double *EB, double dAB, double *W) {
    const int lane = threadIdx.x & 31;
    const int total = nT * d.nPg;
    const float4 *alf = d.alf[c], *alu = d.alfU[c];
    const float *wf = d.wfW[c];
    const double ae[4] = {EA[2] - EA[0], EA[4] - EA[0], EA[3] - EA[1], EA[5] - EA[1]};
    const double be[4] = {EB[2] - EB[0], EB[4] - EB[0], EB[3] - EB[1], EB[5] - EB[1]};
    float ah[4], al[4], bh[4], bl[4];
#pragma unroll
    for (int i = 0; i < 4; i++) {
        ah[i] = (float)ae[i]; al[i] = (float)(ae[i] - (double)ah[i]);
        bh[i] = (float)be[i]; bl[i] = (float)(be[i] - (double)bh[i]);
    }
    const double hexp = -0.5 * P.expo;
    const float hh = (float)(ldexp(rint(ldexp(hexp, 8)), -8));
    const float hl = (float)(hexp - (double)hh);
    const float hf = (float)hexp;
    const float kcd = (float)(P.kc * dAB);
    float Wf[21], Wc[21];
#pragma unroll
    for (int q = 0; q < 21; q++) Wf[q] = Wc[q] = 0.f;
    auto add = [&](int q, float v) {   // Kahan step
        const float y = v - Wc[q];
        const float t = Wf[q] + y;
        Wc[q] = (t - Wf[q]) - y;
        Wf[q] = t;
    };
    for (int idx = lane; idx < total; idx += 32) {
        const float4 a4 = alf[idx], u4 = alu[idx];
        float z0 = fmaf(a4.x, ah[0], fmaf(a4.y, ah[1], fmaf(-a4.z, bh[0], -a4.w * bh[1])));
        float z1 = fmaf(a4.x, ah[2], fmaf(a4.y, ah[3], fmaf(-a4.z, bh[2], -a4.w * bh[3])));
        z0 = fmaf(a4.x, al[0], fmaf(a4.y, al[1], fmaf(-a4.z, bl[0], fmaf(-a4.w, bl[1], z0))));
        z1 = fmaf(a4.x, al[2], fmaf(a4.y, al[3], fmaf(-a4.z, bl[2], fmaf(-a4.w, bl[3], z1))));
        const float r2 = fmaf(z0, z0, z1 * z1);
        int E;
        const float m = frexpf(r2, &E);
        const float t = hh * (float)E;
        const float I = floorf(t);
        const float g = fmaf(hf, log2f(m), fmaf(hl, (float)E, t - I));
        const float f = ldexpf(exp2f(g), (int)I) * wf[idx] * kcd;
        const float px[3] = {1.f - u4.x - u4.y, u4.x, u4.y};
        const float py[3] = {1.f - u4.z - u4.w, u4.z, u4.w};
#pragma unroll
        for (int i = 0; i < 3; i++) {
            const float fx = f * px[i], fy = f * py[i];
#pragma unroll
            for (int j = i; j < 3; j++) {
                add(sym_idx<3>(i, j), fx * px[j]);
                add(6 + sym_idx<3>(i, j), fy * py[j]);
            }
#pragma unroll
            for (int j = 0; j < 3; j++) add(12 + 3 * i + j, fx * py[j]);
        }
    }
#pragma unroll
    for (int q = 0; q < 21; q++) W[q] = (double)Wf[q] - (double)Wc[q];
}

template <bool FAST>
__global__ void __launch_bounds__(128) k_quad_close(QuadArgs a, Duffy d) {
    const int lane = threadIdx.x & 31;
    const long long w = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (w >= a.nlist) return;
    const long long p = a.list[w];
    const int aT = a.pA[p], bT = a.pB[p];
    const ProbParams P = a.probs[a.eprob[aT]];
    const int *aV = &a.T32[(long long)aT * 3];
    const int *bV = &a.T32[(long long)bT * 3];
    // join
    int nEqual = 0, AinB[3] = {0, 0, 0}, BinA[3] = {0, 0, 0}, argA[3], argB[3];
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++)
            if (aV[i] == bV[j]) {
                AinB[i] += 1; BinA[j] += 1;
                argA[nEqual] = i;
                argB[nEqual] = j;
                nEqual++;
            }
    int ia = 0, ib = 0;
    for (int i = 0; i < 3; i++) {
        if (!AinB[i]) { argA[nEqual + ia] = i; ia++; }
        if (!BinA[i]) { argB[nEqual + ib] = i; ib++; }
    }
    double EA[6], EB[6];
    const double *Ea = &a.EC[(long long)aT * 6], *Eb = &a.EC[(long long)bT * 6];
    for (int k = 0; k < 3; k++) {
        int ka = argA[k], kb = argB[k];
        EA[2 * k] = Ea[2 * ka]; EA[2 * k + 1] = Ea[2 * ka + 1];
        EB[2 * k] = Eb[2 * kb]; EB[2 * k + 1] = Eb[2 * kb + 1];
    }
    const double dA = fabs(xsub(xmul(xsub(EA[2], EA[0]), xsub(EA[5], EA[1])), xmul(xsub(EA[3], EA[1]), xsub(EA[4], EA[0]))));
    const double dB = fabs(xsub(xmul(xsub(EB[2], EB[0]), xsub(EB[5], EB[1])), xmul(xsub(EB[3], EB[1]), xsub(EB[4], EB[0]))));
    const int c = nEqual - 1;
    if (c < 0) return;
    const int nT = (nEqual == 1) ? 2 : (nEqual == 2 ? 5 : 6);
    double acc[36];
    for (int i = 0; i < 36; i++) acc[i] = 0;
    if (P.close == MTH_WEAKSING) {
        double W[21];
#pragma unroll
        for (int i = 0; i < 21; i++) W[i] = 0.0;
        if (FAST) weak_accumulate_f32(P, d, c, nT, EA, EB, dA * dB, W);
        else weak_accumulate(P, d, c, nT, EA, EB, dA * dB, W);
#pragma unroll
        for (int i = 0; i < 21; i++) W[i] = warp_sum(W[i]);
        // termLocal[argA a][argA b], termLocalPrime[argB a][argB b], termNonloc and
        // termNonlocPrime [argA a][argB b] (integration.cpp:167-178)
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++) {
                const int sij = i <= j ? sym_idx<3>(i, j) : sym_idx<3>(j, i);
                acc[0 * 9 + 3 * argA[i] + argA[j]] = W[sij];
                acc[2 * 9 + 3 * argB[i] + argB[j]] = W[6 + sij];
                acc[1 * 9 + 3 * argA[i] + argB[j]] = W[12 + 3 * i + j];
                acc[3 * 9 + 3 * argA[i] + argB[j]] = W[12 + 3 * i + j];
            }
    } else {
    const int nLocal = 6 - nEqual, shift = 3 - nEqual;
    // target of (a, b) in the 4 x 9 block vector and its sign
    int tgt[36];
    double sgn[36];
    for (int aa = 0; aa < nLocal; aa++)
        for (int b = 0; b < nLocal; b++) {
            int t;
            double s;
            if (aa < 3) {
                if (b < 3) { t = 0 * 9 + 3 * argA[aa] + argA[b]; s = 1.0; }
                else { t = 1 * 9 + 3 * argA[aa] + argB[b - shift]; s = -1.0; }
            } else {
                if (b < 3) { t = 3 * 9 + 3 * argA[b] + argB[aa - shift]; s = -1.0; }
                else { t = 2 * 9 + 3 * argB[aa - shift] + argB[b - shift]; s = 1.0; }
            }
            tgt[aa * 6 + b] = t;
            sgn[aa * 6 + b] = s;
        }
    // sum over the Duffy points of w pxy pxy^T (symmetric, in registers), then the four blocks
    double M[21];
#pragma unroll
    for (int i = 0; i < 21; i++) M[i] = 0.0;
    if (FAST) {
        if (nEqual == 1) close_accumulate_f32<1>(P, d, c, nT, EA, EB, dA * dB, M);
        else if (nEqual == 2) close_accumulate_f32<2>(P, d, c, nT, EA, EB, dA * dB, M);
        else close_accumulate_f32<3>(P, d, c, nT, EA, EB, dA * dB, M);
    } else {
        if (nEqual == 1) close_accumulate<1, false>(P, d, c, nT, EA, EB, dA * dB, M);
        else if (nEqual == 2) close_accumulate<2, false>(P, d, c, nT, EA, EB, dA * dB, M);
        else close_accumulate<3, false>(P, d, c, nT, EA, EB, dA * dB, M);
    }
#pragma unroll
    for (int i = 0; i < 21; i++) M[i] = warp_sum(M[i]);
    for (int aa = 0; aa < nLocal; aa++)
        for (int b = 0; b < nLocal; b++) acc[tgt[aa * 6 + b]] += sgn[aa * 6 + b] * M[aa <= b ? sym_idx<6>(aa, b) : sym_idx<6>(b, aa)];
    }

    if (a.blocks_out) {
        if (lane == 0) {
            double *o = &a.blocks_out[p * 36];
            for (int i = 0; i < 36; i++) o[i] = acc[i];
            a.ret_out[p] = 1;
        }
        return;
    }
    if (lane == 0) {
        int aVl[3] = {aV[0], aV[1], aV[2]}, bVl[3] = {bV[0], bV[1], bV[2]};
        scatter_blocks<3>(a, aVl, bVl, &acc[0], &acc[9], &acc[18], &acc[27], P.scale_exp, true);
        atomicAdd(a.n_close, 1ULL);
    }
}

}  // namespace nlg
