// Device geometry and model functions of the nonlocal assembly.
//
// The "exact" functions reproduce the reference's FP64 arithmetic operation by operation
// (src/mathhelpers.cpp, src/integration.cpp) with explicit round-to-nearest intrinsics, so that
// no FMA contraction changes a rounding: the interaction predicate they feed decides the sparsity
// pattern and must agree bit for bit with the reference's CPU build.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace nlg {

__device__ __forceinline__ double xadd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double xsub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double xmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double xdiv(double a, double b) { return __ddiv_rn(a, b); }
__device__ __forceinline__ double xsqrt(double a) { return __dsqrt_rn(a); }

// vec_dot / vec_sqL2dist of two 2-vectors (mathhelpers.cpp:255-279): ((0 + a0 b0) + a1 b1)
__device__ __forceinline__ double xdot2(double a0, double a1, double b0, double b1) {
    return xadd(xmul(a0, b0), xmul(a1, b1));
}
__device__ __forceinline__ double xsqdist2(const double *p, const double *x) {
    double d0 = xsub(p[0], x[0]), d1 = xsub(p[1], x[1]);
    return xadd(xmul(d0, d0), xmul(d1, d1));
}

// toPhys(E, p, dim, out) (mathhelpers.cpp:217-225)
template <int DIM>
__device__ __forceinline__ void xtoPhys(const double *E, const double *p, double *x) {
#pragma unroll
    for (int i = 0; i < DIM; i++) {
        double s = xmul(p[0], xsub(E[DIM + i], E[i]));
#pragma unroll
        for (int j = 1; j < DIM; j++) s = xadd(s, xmul(p[j], xsub(E[DIM * (j + 1) + i], E[i])));
        x[i] = xadd(s, E[i]);
    }
}

// signDet(E) of a triangle (mathhelpers.cpp:131-147)
__device__ __forceinline__ double xsignDet2(const double *E) {
    double M00 = xsub(E[2], E[0]), M01 = xsub(E[4], E[0]);
    double M10 = xsub(E[3], E[1]), M11 = xsub(E[5], E[1]);
    double det = xsub(xmul(M00, M11), xmul(M01, M10));
    return det > 0 ? 1.0 : (det < 0 ? -1.0 : 0.0);
}

// absDet(E) of a triangle (mathhelpers.cpp:101-109)
__device__ __forceinline__ double xabsDet2(const double *E) {
    double M00 = xsub(E[2], E[0]), M01 = xsub(E[4], E[0]);
    double M10 = xsub(E[3], E[1]), M11 = xsub(E[5], E[1]);
    return fabs(xsub(xmul(M00, M11), xmul(M01, M10)));
}

// inTriangle (integration.cpp:1283-1298)
__device__ __forceinline__ bool xinTriangle(const double *y, const double *TE, const double *na,
                                            const double *nb, const double *nc) {
    bool a = xdot2(na[0], na[1], xsub(y[0], TE[0]), xsub(y[1], TE[1])) >= 0;
    bool b = xdot2(nb[0], nb[1], xsub(y[0], TE[2]), xsub(y[1], TE[3])) >= 0;
    bool c = xdot2(nc[0], nc[1], xsub(y[0], TE[4]), xsub(y[1], TE[5])) >= 0;
    return a && b && c;
}

// placePointOnCap (integration.cpp:1353-1377); rightNormal (mathhelpers.cpp:74-78)
__device__ __forceinline__ int xplaceCap(const double *ypred, const double *ycur, const double *xc,
                                         double sqdelta, const double *TE, const double *na,
                                         const double *nb, const double *nc, double orientation,
                                         int Rdx, double *R) {
    double n0 = xmul(xsub(ypred[1], ycur[1]), orientation);
    double n1 = xmul(xsub(ycur[0], ypred[0]), orientation);
    double s = xsqrt(xdiv(sqdelta, xdot2(n0, n1, n0, n1)));
    double y[2] = {xadd(xc[0], xmul(n0, s)), xadd(xc[1], xmul(n1, s))};
    if (xinTriangle(y, TE, na, nb, nc)) {
        if (Rdx >= 9) return 0;   // at most 9 polygon points exist; never reached
        R[2 * Rdx] = y[0];
        R[2 * Rdx + 1] = y[1];
        return 1;
    }
    return 0;
}

// method_retriangulate (integration.cpp:1393-1512). Fills the polygon points R (<= 9) of
// B_delta(xc) intersected with the triangle TE and returns their number; the sub-triangles are
// the fan (R0, R[k+1], R[k+2]), k < n-2, present only if n >= 3.
__device__ __forceinline__ int xretriangulate(const double *xc, const double *TE, double sqdelta,
                                              int caps, double *R) {
    int Rdx = 0;
    bool is_onEdge = false, is_firstPointLiesOnVertex = true;
    const double orientation = -xsignDet2(TE);
    double na[2], nb[2], nc[2];
    na[0] = xmul(xsub(TE[3], TE[1]), orientation); na[1] = xmul(xsub(TE[0], TE[2]), orientation);
    nb[0] = xmul(xsub(TE[5], TE[3]), orientation); nb[1] = xmul(xsub(TE[2], TE[4]), orientation);
    nc[0] = xmul(xsub(TE[1], TE[5]), orientation); nc[1] = xmul(xsub(TE[4], TE[0]), orientation);
#pragma unroll 1
    for (int k = 0; k < 3; k++) {
        const double *p = &TE[2 * k];
        const double *q = &TE[2 * (k == 2 ? 0 : k + 1)];
        const double a0 = xsub(q[0], xc[0]), a1 = xsub(q[1], xc[1]);
        const double b0 = xsub(p[0], q[0]), b1 = xsub(p[1], q[1]);
        if (xsqdist2(p, xc) <= sqdelta) {
            if (Rdx < 9) { R[2 * Rdx] = p[0]; R[2 * Rdx + 1] = p[1]; Rdx += 1; }
            is_onEdge = false;
        }
        const double ab = xdot2(a0, a1, b0, b1);
        const double aa = xdot2(a0, a1, a0, a1);
        const double bb = xdot2(b0, b1, b0, b1);
        const double aad = xsub(aa, sqdelta);
        const double v = xsub(xmul(ab, ab), xmul(aad, bb));
        if (v >= 0) {
            const double term1 = xdiv(-ab, bb);
            const double term2 = xdiv(xsqrt(v), bb);
            double lam1, lam2;
            if (term1 > 0) {
                lam1 = xadd(term1, term2);
                lam2 = xdiv(xmul(xdiv(1.0, lam1), aad), bb);
            } else {
                lam2 = xsub(term1, term2);
                lam1 = xdiv(xmul(xdiv(1.0, lam2), aad), bb);
            }
            // the two roots in turn (one code path for both keeps the routine small)
#pragma unroll 1
            for (int qi = 0; qi < 2; qi++) {
                const double lam = qi ? lam2 : lam1;
                bool ok = (0 <= lam) && (lam <= 1);
                if (qi) {
                    const double dl = xsub(lam1, lam2);
                    ok = ok && (xmul(dl, dl) > 0);
                }
                if (!ok) continue;
                const double y[2] = {xadd(xmul(lam, b0), q[0]), xadd(xmul(lam, b1), q[1])};
                is_firstPointLiesOnVertex = is_firstPointLiesOnVertex && (Rdx != 0);
                if (is_onEdge && caps)
                    Rdx += xplaceCap(&R[2 * (Rdx - 1)], y, xc, sqdelta, TE, na, nb, nc, orientation, Rdx, R);
                if (Rdx < 9) { R[2 * Rdx] = y[0]; R[2 * Rdx + 1] = y[1]; Rdx += 1; }
                is_onEdge = true;
            }
        }
    }
    if (is_onEdge && (!is_firstPointLiesOnVertex && Rdx > 1) && caps)
        Rdx += xplaceCap(&R[2 * (Rdx - 1)], &R[0], xc, sqdelta, TE, na, nb, nc, orientation, Rdx, R);
    return Rdx;
}

// placePointCapCenter (integration.cpp:1300-1351): the circular segment of B_delta(xc) cut off by
// the chord (ypred, ycur); its centroid goes to cap if it lies in the triangle, and its area is
// returned (0 otherwise). acos, sin and pow are CUDA's: they may differ from the host's in the
// last bit.
__device__ __forceinline__ double xcap_center(const double *ypred, const double *ycur, const double *xc, double sqdelta,
                                              const double *TE, const double *na, const double *nb, const double *nc,
                                              double orientation, double *cap) {
    const double p1[2] = {xadd(xc[0], xmul(ypred[0], -1.0)), xadd(xc[1], xmul(ypred[1], -1.0))};
    const double p2[2] = {xadd(xc[0], xmul(ycur[0], -1.0)), xadd(xc[1], xmul(ycur[1], -1.0))};
    const double alpha = 0.5 * acos(xdiv(xdot2(p1[0], p1[1], p2[0], p2[1]), sqdelta));
    // rightNormal(ycur, ypred, orientation) (mathhelpers.cpp:74-78)
    const double s0 = xmul(xsub(ypred[1], ycur[1]), orientation), s1 = xmul(xsub(ycur[0], ypred[0]), orientation);
    const double scaling = (4 * sqrt(sqdelta) * pow(sin(alpha), 3)) / (3 * (2 * alpha - sin(2 * alpha))) *
                           sqrt(1. / xdot2(s0, s1, s0, s1));
    const double y[2] = {xadd(xc[0], xmul(s0, scaling)), xadd(xc[1], xmul(s1, scaling))};
    if (xinTriangle(y, TE, na, nb, nc)) {
        cap[0] = y[0];
        cap[1] = y[1];
        return (sqdelta / 2) * (2 * alpha - sin(2 * alpha));
    }
    return 0.0;
}

// method_exact (integration.cpp:1632-1761): the polygon of B_delta(xc) and the triangle without
// cap points (R, n points, as method_retriangulate without caps) and up to three circular
// segments: centroids in caps, areas in capw, their number in *ncaps. A segment counts when its
// area is not within 1e-15 of zero (double_eq, mathhelpers.cpp:370-373).
__device__ __forceinline__ int xmethod_exact(const double *xc, const double *TE, double sqdelta, double *R,
                                             double *caps, double *capw, int *ncaps) {
    int Rdx = 0, nc_ = 0;
    bool is_onEdge = false;
    const double orientation = -xsignDet2(TE);
    double na[2], nb[2], nc[2];
    na[0] = xmul(xsub(TE[3], TE[1]), orientation); na[1] = xmul(xsub(TE[0], TE[2]), orientation);
    nb[0] = xmul(xsub(TE[5], TE[3]), orientation); nb[1] = xmul(xsub(TE[2], TE[4]), orientation);
    nc[0] = xmul(xsub(TE[1], TE[5]), orientation); nc[1] = xmul(xsub(TE[4], TE[0]), orientation);
#pragma unroll 1
    for (int k = 0; k < 3; k++) {
        const double *p = &TE[2 * k];
        const double *q = &TE[2 * (k == 2 ? 0 : k + 1)];
        const double a0 = xsub(q[0], xc[0]), a1 = xsub(q[1], xc[1]);
        const double b0 = xsub(p[0], q[0]), b1 = xsub(p[1], q[1]);
        if (xsqdist2(p, xc) <= sqdelta) {
            if (Rdx < 9) { R[2 * Rdx] = p[0]; R[2 * Rdx + 1] = p[1]; Rdx += 1; }
            is_onEdge = false;
        }
        const double ab = xdot2(a0, a1, b0, b1);
        const double aa = xdot2(a0, a1, a0, a1);
        const double bb = xdot2(b0, b1, b0, b1);
        const double aad = xsub(aa, sqdelta);
        const double v = xsub(xmul(ab, ab), xmul(aad, bb));
        if (v >= 0) {
            const double term1 = xdiv(-ab, bb);
            const double term2 = xdiv(xsqrt(v), bb);
            double lam1, lam2;
            if (term1 > 0) {
                lam1 = xadd(term1, term2);
                lam2 = xdiv(xmul(xdiv(1.0, lam1), aad), bb);
            } else {
                lam2 = xsub(term1, term2);
                lam1 = xdiv(xmul(xdiv(1.0, lam2), aad), bb);
            }
#pragma unroll 1
            for (int qi = 0; qi < 2; qi++) {
                const double lam = qi ? lam2 : lam1;
                bool ok = (0 <= lam) && (lam <= 1);
                if (qi) {
                    const double dl = xsub(lam1, lam2);
                    ok = ok && (xmul(dl, dl) > 0);
                }
                if (!ok) continue;
                const double y[2] = {xadd(xmul(lam, b0), q[0]), xadd(xmul(lam, b1), q[1])};
                if (is_onEdge && nc_ < 3) {
                    capw[nc_] = xcap_center(&R[2 * (Rdx - 1)], y, xc, sqdelta, TE, na, nb, nc, orientation, &caps[2 * nc_]);
                    nc_ += !(fabs(capw[nc_]) < 1e-15);
                }
                if (Rdx < 9) { R[2 * Rdx] = y[0]; R[2 * Rdx + 1] = y[1]; Rdx += 1; }
                is_onEdge = true;
            }
        }
    }
    if (is_onEdge && nc_ < 3) {
        capw[nc_] = xcap_center(&R[2 * (Rdx - 1)], &R[0], xc, sqdelta, TE, na, nb, nc, orientation, &caps[2 * nc_]);
        nc_ += !(fabs(capw[nc_]) < 1e-15);
    }
    *ncaps = nc_;
    return Rdx;
}

// baryCenter(dim, E) (mathhelpers.cpp:184-196) and method_baryCenter (integration.cpp:1262-1280):
// true iff |x - bary(T)|^2 <= delta^2.
template <int DIM>
__device__ __forceinline__ void xbary(const double *E, double *b) {
#pragma unroll
    for (int j = 0; j < DIM; j++) {
        double s = E[j];
#pragma unroll
        for (int i = 1; i <= DIM; i++) s = xadd(s, E[DIM * i + j]);
        b[j] = xdiv(s, (double)(DIM + 1));
    }
}
// Per-element barycenter as a double-float pair, for the FP32 barycenter tests: DIM hi floats at
// offset 0 and DIM lo floats at offset BC_STRIDE / 2 (3D pads each half to four floats).
template <int DIM>
constexpr int BC_STRIDE = DIM == 2 ? 4 : 8;

// Offset of element b's barycenter from the outer element's first vertex (ohi + olo), in FP32:
// the difference of two double-float pairs, like the vertex offsets.
template <int DIM>
__device__ __forceinline__ void bary_offset(const float *BCf, long long b, const float *ohi, const float *olo,
                                            float *bf) {
    const float4 *q = reinterpret_cast<const float4 *>(BCf + b * BC_STRIDE<DIM>);
    if (DIM == 2) {
        const float4 v = q[0];
        bf[0] = (v.x - ohi[0]) + (v.z - olo[0]);
        bf[1] = (v.y - ohi[1]) + (v.w - olo[1]);
    } else {
        const float4 h = q[0], l = q[1];
        bf[0] = (h.x - ohi[0]) + (l.x - olo[0]);
        bf[1] = (h.y - ohi[1]) + (l.y - olo[1]);
        bf[DIM - 1] = (h.z - ohi[DIM - 1]) + (l.z - olo[DIM - 1]);
    }
}

template <int DIM>
__device__ __forceinline__ bool xbaryInside(const double *x, const double *b, double sqdelta) {
    double d = xsub(x[0], b[0]);
    double r = xmul(d, d);
#pragma unroll
    for (int j = 1; j < DIM; j++) {
        d = xsub(x[j], b[j]);
        r = xadd(r, xmul(d, d));
    }
    return !(r > sqdelta);
}

// solve2x2 (mathhelpers.cpp:41-71). Returns false where the reference aborts.
__device__ __forceinline__ bool xsolve2x2(const double *A, const double *b, double *x) {
    int dx0 = 0, dx1 = 1;
    if (fabs(A[0]) < fabs(A[2])) { dx0 = 1; dx1 = 0; }
    if (fabs(A[2 * dx0]) < 1e-15) return false;
    const double l = xdiv(A[2 * dx1], A[2 * dx0]);
    const double u = xsub(A[2 * dx1 + 1], xmul(l, A[2 * dx0 + 1]));
    if (u == 0) return false;
    x[1] = xdiv(xsub(b[dx1], xmul(l, b[dx0])), u);
    x[0] = xdiv(xsub(b[dx0], xmul(A[2 * dx0 + 1], x[1])), A[2 * dx0]);
    return true;
}

// toRef (mathhelpers.cpp:227-240)
__device__ __forceinline__ bool xtoRef(const double *E, const double *y, double *p) {
    double M[4] = {xsub(E[2], E[0]), xsub(E[4], E[0]), xsub(E[3], E[1]), xsub(E[5], E[1])};
    double b[2] = {xsub(y[0], E[0]), xsub(y[1], E[1])};
    return xsolve2x2(M, b, p);
}

// ------------------------------------------------------------------- model (model.cpp)
// KER_LABELED .. KER_CONSTTRUNC depend on the elements' labels or on absolute positions: FP64
// passes only.
// KER_CONSTFIELD .. KER_MICROFIELD3D are matrix-valued (outdim 2, 2, 3): the vector path only.
enum KernelId {
    KER_CONSTANT = 0, KER_PARABOLA = 1, KER_FRACTIONAL = 2, KER_CONSTANT3D = 3,
    KER_LABELED = 4, KER_NOTCH = 5, KER_LABELEDNOTCH = 6, KER_LABELEDVALVE = 7, KER_CONSTTRUNC = 8,
    KER_CONSTFIELD = 9, KER_MICROFIELD = 10, KER_MICROFIELD3D = 11
};
// MTH_RETRI_UNSYMM .. MTH_NOTRUNC: 2D, FP64 passes only.
enum MethodId {
    MTH_RETRIANGULATE = 0, MTH_BARYCENTER = 1, MTH_FRACTIONAL = 2, MTH_RETRI_UNSYMM = 3, MTH_SUBSET = 4,
    MTH_AVERAGE = 5, MTH_BARY_RT = 6, MTH_NOTRUNC = 7, MTH_WEAKSING = 8, MTH_EXACT = 9
};
// LOAD_LINEARFIELD .. LOAD_BOTHFIELD are vector-valued (outdim 2, except LOAD_LINEARFIELD3D: 3).
enum LoadId {
    LOAD_LINEAR = 0, LOAD_LINEAR3D = 1, LOAD_CONSTANT = 2, LOAD_GAUSSIAN = 3, LOAD_JUMP = 4, LOAD_TENSORSIN = 5,
    LOAD_LINEARFIELD = 6, LOAD_LINEARFIELD3D = 7, LOAD_RIGHTFIELD = 8, LOAD_DOWNFIELD = 9, LOAD_BOTHFIELD = 10
};

// Per-problem parameters (one entry per independent assembly).
struct ProbParams {
    double sqdelta, delta;
    double kc;       // kernel constant (host-computed with the reference's formula)
    double kc2;      // labeled kernel: the constant of the label >= 21 branch
    double expo;     // fractional: dim + 2s
    float sqdelta_f, kc_f, expo_f, pad_f;
    int kernel, remote, close, caps;
    int full_search, singular, load, scale_exp;
    int elem_off, nE, vert_off, nV;
    int bridges;          // the mesh has label-0 elements (searched through, never paired)
    int zeta;             // domain-decomposition weights 1 / zeta on every pair
    double fx_unit;   // value of one unit of the 64-bit fixed-point CSR sums: 2^fx_ue
    float fx_mul;     // 2^-fx_ue
    int fx_ue;        // scale_exp + guard bits - 62
    double el;        // mean element measure (bounding box / nE), for capacity estimates
};

// Close pairs of a singular kernel take a Duffy rule: fractional or weakSingular.
__host__ __device__ __forceinline__ bool duffy_close(const ProbParams &P) {
    return P.singular && (P.close == MTH_FRACTIONAL || P.close == MTH_WEAKSING);
}

// FP64 kernel value k(x, lx, y, ly), lx and ly the labels of the elements of x and y
// (model.cpp:25-28, 36-42, 52-60, 62-65, 67-114, 126-138). Where the reference aborts (labeled:
// |x - y| >= delta, or 10 lx + ly in 14..20) it sets err[7] and returns 0.
template <int DIM>
__device__ __forceinline__ double kernel_f64(const ProbParams &P, const double *x, long long lx, const double *y,
                                             long long ly, int *err) {
    switch (P.kernel) {
    case KER_LABELED: {
        const double z0 = xsub(x[0], y[0]), z1 = xsub(x[1], y[1]);
        const double dist = xadd(xmul(z0, z0), xmul(z1, z1));
        const long long label = 10 * lx + ly;
        if (dist >= P.sqdelta || (label > 13 && label < 21)) { atomicOr(&err[7], 1); return 0.0; }
        if (label <= 12) return P.kc;
        if (label >= 21) return P.kc2 * (1 - dist / P.sqdelta);
        return 0.0;
    }
    case KER_NOTCH: {   // zero across the notch {x1 = 0, x0 > 0}
        const bool cross = ((x[1] > 0) != (y[1] > 0)) && x[0] > 0 && y[0] > 0;
        return cross ? 0.0 : P.kc;
    }
    case KER_LABELEDNOTCH: return lx + ly == 7 ? 0.0 : P.kc;
    case KER_LABELEDVALVE: return lx >= ly ? P.kc : 0.0;
    case KER_CONSTTRUNC: {
        const double z0 = xsub(x[0], y[0]), z1 = xsub(x[1], y[1]);
        return P.sqdelta > xadd(xmul(z0, z0), xmul(z1, z1)) ? P.kc : 0.0;
    }
    case KER_PARABOLA: {
        double z0 = x[0] - y[0], z1 = x[1] - y[1];
        return P.kc * (P.sqdelta - (z0 * z0 + z1 * z1));
    }
    case KER_FRACTIONAL: {
        double r = 0;
#pragma unroll
        for (int i = 0; i < DIM; i++) { double z = x[i] - y[i]; r += z * z; }
        return P.kc * (1.0 / pow(sqrt(r), P.expo));
    }
    default:
        return P.kc;
    }
}

// FP32 kernel value from the difference z = x - y (local coordinates).
__device__ __forceinline__ float kernel_f32(const ProbParams &P, float z0, float z1) {
    switch (P.kernel) {
    case KER_PARABOLA:
        return P.kc_f * (P.sqdelta_f - (z0 * z0 + z1 * z1));
    case KER_FRACTIONAL: {
        float r2 = z0 * z0 + z1 * z1;
        return P.kc_f * exp2f(-0.5f * P.expo_f * log2f(r2));
    }
    default:
        return P.kc_f;
    }
}

// Scalar load functions (model.cpp:201-203, 240-261). gaussian and tensorsin call CUDA's exp and
// sin, which may differ from the host's in the last bit.
__device__ __forceinline__ double load_f64(int load, const double *x) {
    switch (load) {
    case LOAD_LINEAR: return -2. * (x[1] + 1.);
    case LOAD_LINEAR3D: return -2. * (x[1] + 2.);
    case LOAD_GAUSSIAN: {
        const double a = x[0] * x[0], b = x[1] * x[1];
        return -4. * (a + b - 1.) * exp(-a - b);
    }
    case LOAD_JUMP: return (x[0] + x[1] - 0.5 > -1e-15) ? -4. : 4.;   // EPSILON of mathhelpers.h:11
    case LOAD_TENSORSIN: return 32. * (M_PI * M_PI) * sin(x[0] * M_PI * 4) * sin(x[1] * M_PI * 4);
    default: return 1.0;
    }
}

// Vector load functions (model.cpp:204-238): the components f_o(x).
__device__ __forceinline__ void load_vec_f64(int load, const double *x, double *f) {
    const double c = M_PI / 2.0;
    switch (load) {
    case LOAD_LINEARFIELD: f[0] = -c * (1.0 + 2 * x[0]); f[1] = -c * x[1]; break;
    case LOAD_LINEARFIELD3D:
        f[0] = -c * (1.0 + 2 * x[0]) * x[1] * x[1]; f[1] = -c * x[1] * x[1]; f[2] = -c * x[2] * x[1] * x[1]; break;
    case LOAD_RIGHTFIELD: f[0] = 1.0e-1; f[1] = 0.0; break;
    case LOAD_DOWNFIELD: f[0] = 0.0; f[1] = -M_PI * 2; break;
    case LOAD_BOTHFIELD: f[0] = -M_PI; f[1] = -M_PI * 2; break;
    default: f[0] = load_f64(load, x); break;
    }
}

// Matrix-valued kernels (model.cpp:140-191), kv[OD * aOut + bOut] of z = x - y; P.kc holds
// 4 / (pi delta^4) (constantField) or 3 / delta^3 (the microelastic fields).
template <int OD>
__device__ __forceinline__ void kernel_field_f64(const ProbParams &P, const double *x, const double *y, double *kv) {
    if (P.kernel == KER_CONSTFIELD) {   // [k(0,0), k(0,1), k(1,0), k(1,1)] = [c, 0, c, 0]
        kv[0] = P.kc; kv[1] = 0.0; kv[2] = P.kc; kv[3] = 0.0;
        return;
    }
    double z[3] = {0, 0, 0}, r2 = 0;
#pragma unroll
    for (int i = 0; i < OD; i++) { z[i] = x[i] - y[i]; r2 += z[i] * z[i]; }
    const double r = sqrt(r2);
    const double cd = P.kc * (1.0 / (r * r * r));
#pragma unroll
    for (int i = 0; i < OD; i++)
#pragma unroll
        for (int j = 0; j < OD; j++) kv[OD * i + j] = cd * z[i] * z[j];
}

}  // namespace nlg
