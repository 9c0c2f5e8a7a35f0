// Certified FP32 ball-triangle geometry.
//
// GB300 executes FP64 at a small fraction of its FP32 rate, so the interaction geometry runs in
// FP32 on coordinates relative to the ball center, and every discrete decision of the
// reference's method_retriangulate (integration.cpp:1393-1512) - vertex inside the ball,
// discriminant sign, root in [0, 1], cap point inside the triangle, orientation - is checked
// against a margin far above the FP32 rounding error of its operands. When every decision clears
// its margin, the FP32 run takes exactly the branches the FP64 reference takes (same polygon,
// same point count) and its points agree to FP32 accuracy; otherwise the caller reruns the
// exact FP64 routine (geometry.cuh). The sparsity pattern therefore stays bit-exact while FP64
// runs only for near-tangent and near-degenerate cuts.
#pragma once
#include <cuda_runtime.h>

namespace nlg {

// Margins, relative to the magnitude of each decision's operands. The FP32 rounding error of a
// tested quantity is a bounded number of units of 2^-24 of that magnitude (coordinates are local
// to the outer element, built from double-float differences); each margin is 256 or more such
// units, and the bound for the vertex tests is written out below MIX_MAX_H_OVER_DELTA.
// Which roots of |q + l (p - q) - x|^2 = delta^2 lie in [0, 1] is fixed by the signs of its values
// at 0 and 1 (vertex distances, MARG_D) and of the discriminant (MARG_V, flagged only when the
// tangent point lies near the segment); MARG_L additionally guards the computed roots.
constexpr float MARG_D = 1.0f / 65536.0f;  // |d^2 - delta^2| <= MARG_D * delta^2: vertex on the sphere
constexpr float MARG_V = 1.0f / 16384.0f;  // |disc| <= MARG_V * (ab^2 + aa*bb): near-tangent line
constexpr float MARG_L = 1.0f / 16384.0f;  // root within MARG_L of 0 or 1
constexpr float MARG_C = 1.0f / 65536.0f;  // cap point near a triangle edge line
constexpr float MARG_O = 1.0f / 4096.0f;   // near-degenerate triangle

struct F2 {
    float x, y;
};
__device__ __forceinline__ F2 f2(float x, float y) { return F2{x, y}; }
__device__ __forceinline__ F2 operator-(F2 a, F2 b) { return F2{a.x - b.x, a.y - b.y}; }
__device__ __forceinline__ F2 operator+(F2 a, F2 b) { return F2{a.x + b.x, a.y + b.y}; }
__device__ __forceinline__ float dot(F2 a, F2 b) { return fmaf(a.x, b.x, a.y * b.y); }

constexpr float U32 = 5.9604645e-8f;      // 2^-24

// Error bound of the squared distances the vertex tests compare (u = 2^-24). Coordinates are local
// to the outer element T's first vertex: an outer point lies within h (T's diameter) of it, and a
// candidate element's vertices within delta + 3h (h the largest diameter). A vertex offset (and a
// barycenter offset, from the barycenter's own double-float pair) is the FP32 difference of
// double-float (hi + lo) pairs, |error| <= 2.01 u (delta + 3h); the outer point's
// offset is one FP32 rounding, <= u h; their difference Q adds u |Q|. At |Q| ~ delta the squared
// distance Q.Q (one FMA, 2u) is then off by at most
//   2 delta (u delta + 2.01 u (delta + 3.5 h)) + 2 u delta^2 = u delta^2 (8.02 + 14.07 h / delta),
// below MARG_D delta^2 = 256 u delta^2 while h <= 17.6 delta. The mixed path therefore refuses
// meshes with an element diameter above MIX_MAX_H_OVER_DELTA delta. The bounding-disc tests of the
// pair search (centroid distance against (delta +- r)^2) have the same bound divided by
// (1 + r / delta)^2, with r inflated by 8u.
constexpr double MIX_MAX_H_OVER_DELTA = 16.0;

// inTriangle with margin: y carries a position error bound ey; a sign test is ambiguous when its
// value is within twice the bound on its error.
__device__ __forceinline__ bool fin_triangle(F2 y, float ey, const F2 *P, const F2 *nu, bool &amb, unsigned *why = nullptr) {
    bool in = true;
#pragma unroll
    for (int e = 0; e < 3; e++) {
        F2 w = y - P[e];
        float s = dot(nu[e], w);
        const float nn = fabsf(nu[e].x) + fabsf(nu[e].y);
        const float err = nn * (ey + 8.f * U32 * (fabsf(w.x) + fabsf(w.y) + fabsf(y.x) + fabsf(y.y)));
        if (fabsf(s) <= fmaxf(2.f * err, MARG_C * nn * (fabsf(w.x) + fabsf(w.y)))) { amb = true; if (why) *why |= (ey > 16.f * U32 * (fabsf(y.x) + fabsf(y.y)) ? 64u : 32u); }
        in = in && (s >= 0.f);
    }
    return in;
}

// Polygon point bookkeeping: the positions go to the caller's array; the error bounds of a
// point (across its edge line: rounding; along it: root error, large near tangency) are needed
// only for the caps next to the last and the first point, so only those two are kept.
struct FPt {
    F2 y;
    float eperp, ealong;
};

struct FPoly {
    F2 *R;     // points, at most 9
    int n;
    FPt first, last;
};

__device__ __forceinline__ void fpush(FPoly &Y, const FPt &p, bool &amb) {
    if (Y.n >= 9) { amb = true; return; }
    if (Y.R) Y.R[Y.n] = p.y;   // null R: the count only
    if (Y.n == 0) Y.first = p;
    Y.last = p;
    Y.n++;
}

// Cap point between two consecutive polygon points (placePointOnCap, integration.cpp:1353-1377),
// appended when it lies in the triangle. The reference places it at x + delta * n / |n| with n the
// oriented normal of the chord. Both chord ends are cut points on the sphere, so in exact
// arithmetic that point is also delta * m / |m| with m the chord midpoint (the perpendicular
// bisector of a chord passes through the center), on the side sign(n . m). This form turns the
// chord ends' position errors into a cap error of the same size instead of amplifying them by
// delta / |chord|.
__device__ __forceinline__ void fplace_cap(FPoly &Y, const FPt &a, const FPt &b, float sq, const F2 *P,
                                           const F2 *nu, float orientation, bool &amb, unsigned *why = nullptr) {
    const F2 n = f2((a.y.y - b.y.y) * orientation, (b.y.x - a.y.x) * orientation);
    const F2 m = f2(0.5f * (a.y.x + b.y.x), 0.5f * (a.y.y + b.y.y));
    const float mm = dot(m, m), nn = dot(n, n);
    const float nm = dot(n, m);
    const float delta = sqrtf(sq);
    // n and m are parallel up to rounding; a near-diametral chord (m ~ 0) is left to FP64
    if (!(nm * nm > 0.25f * nn * mm) || mm <= 1e-6f * sq) { amb = true; if (why) *why |= 128u; return; }
    const float s = (nm > 0.f ? delta : -delta) * rsqrtf(mm);
    const F2 y = f2(m.x * s, m.y * s);
    const float em = 0.5f * (a.eperp + a.ealong + b.eperp + b.ealong);
    const float ey = delta * em * rsqrtf(mm) + em + 8.f * U32 * delta;
    if (fin_triangle(y, ey, P, nu, amb, why)) fpush(Y, FPt{y, ey, 0.f}, amb);
}

// FP32 method_retriangulate with the triangle P given relative to the ball center. Returns the
// polygon point count (sub-triangles: fan (R0, R[j+1], R[j+2])); amb = true when a decision was
// within its margin (the result must then be recomputed in FP64). With R null only the count is
// kept (the interaction test of the pair search).
__device__ __forceinline__ int fretriangulate(const F2 *P, float sq, int caps, F2 *R, bool &amb,
                                              unsigned *why = nullptr) {
    FPoly Y;
    Y.R = R;
    Y.n = 0;
    bool is_onEdge = false, is_firstPointLiesOnVertex = true;
    const F2 e1 = P[1] - P[0], e2 = P[2] - P[0];
    const float det = e1.x * e2.y - e1.y * e2.x;
    if (fabsf(det) <= MARG_O * (fabsf(e1.x) + fabsf(e1.y)) * (fabsf(e2.x) + fabsf(e2.y))) { amb = true; if (why) *why |= 1u; }
    const float orientation = det > 0 ? -1.f : 1.f;
    F2 nu[3];
#pragma unroll
    for (int e = 0; e < 3; e++) {
        F2 a = P[e], b = P[e == 2 ? 0 : e + 1];
        nu[e] = f2((b.y - a.y) * orientation, (a.x - b.x) * orientation);
    }
    const float sqlo = sq * (1.f - MARG_D), sqhi = sq * (1.f + MARG_D);
#pragma unroll 1
    for (int k = 0; k < 3; k++) {
        const F2 p = P[k], q = P[k == 2 ? 0 : k + 1];
        const F2 b = p - q;
        const float dp = dot(p, p);
        if (dp > sqlo && dp < sqhi) { amb = true; if (why) *why |= 2u; }
        if (dp <= sq) {
            fpush(Y, FPt{p, 4.f * U32 * (fabsf(p.x) + fabsf(p.y)), 0.f}, amb);
            is_onEdge = false;
        }
        const float ab = dot(q, b), aa = dot(q, q), bb = dot(b, b);
        const float aad = aa - sq;
        if (fabsf(aad) <= MARG_D * sq) { amb = true; if (why) *why |= 2u; }   // q on the sphere (f(0) ~ 0)
        const float v = ab * ab - aad * bb;
        const float vscale = ab * ab + aa * bb;
        if (fabsf(v) <= MARG_V * vscale) {
            // near-tangent line: only ambiguous if a root can fall near the segment [0, 1]
            const float t = -ab / bb;
            const float r = sqrtf(2.f * MARG_V * vscale) / bb;
            if (t + r >= -MARG_L && t - r <= 1.f + MARG_L) { amb = true; if (why) *why |= 4u; }
        }
        if (v >= 0.f) {
            const float sv = sqrtf(v);
            const float term1 = -ab / bb;
            const float term2 = sv / bb;
            float lam1, lam2;
            if (term1 > 0.f) {
                lam1 = term1 + term2;
                lam2 = aad / (bb * lam1);
            } else {
                lam2 = term1 - term2;
                lam1 = aad / (bb * lam2);
            }
            // cut point error: across the edge line only rounding; along it the root moves by
            // err(v) / (2 sqrt(v) |b|), and err(v) <= 10 u (ab^2 + aa bb) (two products of dot
            // products, each within a few u of its magnitude); bound taken twice
            const float eperp = 8.f * U32 * (fabsf(q.x) + fabsf(q.y) + fabsf(b.x) + fabsf(b.y));
            const float ealong = 10.f * U32 * vscale / fmaxf(sv * sqrtf(bb), 1e-30f);
            if (fabsf(lam1) <= MARG_L || fabsf(lam1 - 1.f) <= MARG_L) { amb = true; if (why) *why |= 8u; }
            if (fabsf(lam2) <= MARG_L || fabsf(lam2 - 1.f) <= MARG_L) { amb = true; if (why) *why |= 16u; }
            // the two roots in turn (one code path for both keeps the routine small)
#pragma unroll 1
            for (int qi = 0; qi < 2; qi++) {
                const float lam = qi ? lam2 : lam1;
                if (!(lam >= 0.f && lam <= 1.f && (qi == 0 || v > 0.f))) continue;
                is_firstPointLiesOnVertex = is_firstPointLiesOnVertex && (Y.n != 0);
                const FPt y{f2(fmaf(lam, b.x, q.x), fmaf(lam, b.y, q.y)), eperp, ealong};
                if (is_onEdge && caps) fplace_cap(Y, Y.last, y, sq, P, nu, orientation, amb, why);
                fpush(Y, y, amb);
                is_onEdge = true;
            }
        }
    }
    if (is_onEdge && (!is_firstPointLiesOnVertex && Y.n > 1) && caps) {
        const FPt last = Y.last, first = Y.first;
        fplace_cap(Y, last, first, sq, P, nu, orientation, amb, why);
    }
    return Y.n;
}

// True when the segment [p, q] stays farther than sqrt(lim) from the origin (end points given
// farther already). The closest point is an end point unless the origin projects inside the
// segment, where the squared distance is (p x u)^2 / |u|^2: compared multiplied by |u|^2, so no
// division is needed (the cross product keeps its relative accuracy near the threshold).
__device__ __forceinline__ bool fseg_far(F2 p, F2 q, float lim) {
    const F2 u = q - p;
    const float uu = dot(u, u), pu = dot(p, u);
    if (!(pu < 0.f && -pu < uu)) return true;   // the closest point is an end point
    const float cr = fmaf(p.x, u.y, -p.y * u.x);
    return cr * cr > lim * uu;
}

enum { CLS_OUT = 0, CLS_IN = 1, CLS_CUT = 2 };

// Fast classes of one outer point against a triangle (relative to the ball center):
//   CLS_IN   all vertices inside with margin: the polygon is the triangle itself
//   CLS_OUT  every edge farther than delta with margin: no polygon point at all
//   CLS_CUT  anything else
__device__ __forceinline__ int fclassify(const F2 *P, float sq) {
    const float sqlo = sq * (1.f - MARG_D), sqhi = sq * (1.f + MARG_D);
    const float d0 = dot(P[0], P[0]), d1 = dot(P[1], P[1]), d2 = dot(P[2], P[2]);
    if (d0 < sqlo && d1 < sqlo && d2 < sqlo) return CLS_IN;
    const float m = fminf(fminf(d0, d1), d2);
    if (m > sqhi) {
        if (fseg_far(P[0], P[1], sqhi) && fseg_far(P[1], P[2], sqhi) && fseg_far(P[2], P[0], sqhi)) return CLS_OUT;
    }
    return CLS_CUT;
}

}  // namespace nlg
