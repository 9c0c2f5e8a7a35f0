// nlfem oracle: CPU restatement of the reference assembly path (TEST INFRASTRUCTURE ONLY).
//
// This file is the checker for the GPU library, never a product path. Only tests/, the smoke
// check and bench.py's CPU-baseline / reference arm load it. It restates, function by function,
// the reference's FP64 algorithm for nonlocal stiffness-matrix and load-vector assembly
// (cagau/nlfem). Every function cites the reference file:line it follows. Arithmetic keeps the
// reference's operation order; it is compiled with -ffp-contract=off so no FMA contraction
// changes a rounding (the reference's x86 build has none either).
//
// Parity status: the reference's own tests hold no golden vectors for the assembled matrix or
// load vector, and the reference itself cannot be built here (it needs Armadillo, METIS and
// CGAL, none of which exist in this image). Parity of this restatement is therefore UNPINNED
// for the assembled values; it is pinned only where fixtures exist (quadrature tables, tensor
// Gauss rule, vertex labels, arma file format, 6-tet split). See the oracle tests.
//
// Differences from the reference that cannot change results beyond rounding:
//  * arma::det is replaced by the cofactor formula (feeds |det| only, never a predicate).
//  * METIS_MeshToDual is replaced by a sorted vertex-sharing adjacency (the BFS pair set does
//    not depend on adjacency order; only the map's summation order may).
//  * METIS_PartMeshDual (thread split) is replaced by contiguous element blocks.

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <queue>
#include <string>
#include <vector>
#include <algorithm>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

const double EPSILON = 1e-15;        // mathhelpers.h:11
const double SCALEDET = 0.0625;      // integration.cpp:44, MeshTypes.cpp:257

enum KernelId { K_CONSTANT = 0, K_PARABOLA = 1, K_FRACTIONAL = 2, K_CONSTANT3D = 3, K_LABELED = 4, K_NOTCH = 5,
                K_LABELEDNOTCH = 6, K_LABELEDVALVE = 7, K_CONSTTRUNC = 8, K_LINPROTO = 9,
                K_FIELD_CONST = 10, K_FIELD_PROTO = 11, K_FIELD_PROTO3D = 12, K_CONSTLINF = 13, K_NONE = -1 };
enum LoadId { F_LINEAR = 0, F_LINEAR3D = 1, F_CONSTANT = 2, F_GAUSSIAN = 3, F_JUMP = 4, F_TENSORSIN = 5,
              F_FIELD_LINEAR = 6, F_FIELD_LINEAR3D = 7, F_FIELD_RIGHT = 8, F_FIELD_DOWN = 9, F_FIELD_BOTH = 10,
              F_NONE = -1 };
enum MethodId { M_RETRIANGULATE = 0, M_BARYCENTER = 1, M_FRACTIONAL = 2, M_RETRI_UNSYMM = 3, M_SUBSET = 4,
                M_AVERAGE = 5, M_BARY_RT = 6, M_NOTRUNC = 7, M_WEAKSING = 8, M_EXACT = 9, M_RETRI_LINF = 10,
                M_UNSYMM_LINF = 11, M_NONE = -1 };

struct Mesh {
    int dim, dV, outdim, is_dg;
    long nE, nV, K;
    const long *T, *labT, *labV;
    const double *V;
    double sqdelta, delta, frac_s;
    int kernel, load;
    int remote, close;   // MethodId of integrate_remote / integrate_close
    int is_singular;
    int caps, full_search;
    int linf = 0;        // the retriangulate rules use the L-infinity ball (Cassemble.cpp:134-141)
    // domain decomposition (Cassemble.cpp:649-657): element -> subdomain indicator, CSR
    const long *zeta_indices = nullptr, *zeta_indptr = nullptr;
    long nZeta = 0;
};

struct Quad {
    const double *Px, *dx, *Py, *dy;
    int nPx, nPy;
    std::vector<double> psix, psiy;  // column-major (dV, nP): psi[dV*k + a]
    int nPg;
    const double *dg;
    // Duffy tables of the fractional close-pair rule, index [case][ (t*nPg + k)*4 + j ]
    std::vector<double> alphaC[3], tdetFrac[3];
    // weakSingular: the points with xi kept (alpha) and the determinant with xi^(1 - 2s)
    std::vector<double> alphaU[3], tdetWeak[3];
};

struct Elem {
    double E[12];
    double absDet;
    long label;
    long Tdx;
};

// ---------------------------------------------------------------- math helpers (mathhelpers.cpp)
inline double absolute(double v) { return v < 0 ? -v : v; }                // mathhelpers.cpp:362-368
inline bool double_eq(double x, double y, double eps = EPSILON) {           // mathhelpers.cpp:370-373
    return absolute(x - y) < eps;
}
inline double sq(double v) { return v * v; }  // pow(v, 2): gcc folds pow(x, 2.0) to x*x

double vec_dot(const double *x, const double *y, int len) {                 // mathhelpers.cpp:255-263
    double r = 0;
    for (int i = 0; i < len; i++) r += x[i] * y[i];
    return r;
}
double vec_sqL2dist(const double *x, const double *y, int len) {            // mathhelpers.cpp:272-279
    double r = 0;
    for (int i = 0; i < len; i++) r += sq(x[i] - y[i]);
    return r;
}

int solve2x2(const double *A, const double *b, double *x) {                 // mathhelpers.cpp:41-71
    int dx0 = 0, dx1 = 1;
    if (absolute(A[0]) < absolute(A[2])) { dx0 = 1; dx1 = 0; }
    if (double_eq(A[2 * dx0], 0)) return -1;  // reference aborts
    double l = A[2 * dx1] / A[2 * dx0];
    double u = A[2 * dx1 + 1] - l * A[2 * dx0 + 1];
    if (u == 0) return -1;                     // reference aborts
    x[1] = (b[dx1] - l * b[dx0]) / u;
    x[0] = (b[dx0] - A[2 * dx0 + 1] * x[1]) / A[2 * dx0];
    return 0;
}

void rightNormal(const double *y0, const double *y1, double orientation, double *n) {  // :74-78
    n[0] = y1[1] - y0[1];
    n[1] = y0[0] - y1[0];
    n[0] = n[0] * orientation;
    n[1] = n[1] * orientation;
}

double absDet2(const double *E) {                                          // mathhelpers.cpp:101-109
    double M00 = E[2] - E[0], M01 = E[4] - E[0];
    double M10 = E[3] - E[1], M11 = E[5] - E[1];
    return absolute(M00 * M11 - M01 * M10);
}

double detDim(const double *E, int dim) {
    // mathhelpers.cpp:112-129: M(j, i-1) = E[j + dim*i] - E[j]; arma::det(M) (cofactor form here)
    if (dim == 2) {
        double a = E[2] - E[0], b = E[4] - E[0];
        double c = E[3] - E[1], d = E[5] - E[1];
        return a * d - c * b;
    }
    double M[3][3];
    for (int i = 1; i < 4; i++)
        for (int j = 0; j < 3; j++) M[j][i - 1] = E[j + 3 * i] - E[j];
    return M[0][0] * (M[1][1] * M[2][2] - M[1][2] * M[2][1])
         - M[0][1] * (M[1][0] * M[2][2] - M[1][2] * M[2][0])
         + M[0][2] * (M[1][0] * M[2][1] - M[1][1] * M[2][0]);
}
double absDetDim(const double *E, int dim) { return absolute(detDim(E, dim)); }

double signDet2(const double *E) {                                         // mathhelpers.cpp:131-147
    double M00 = E[2] - E[0], M01 = E[4] - E[0];
    double M10 = E[3] - E[1], M11 = E[5] - E[1];
    double det = M00 * M11 - M01 * M10;
    if (det > 0) return 1.;
    if (det < 0) return -1.;
    return 0.0;
}

void baryCenter(int dim, const double *E, double *bary) {                  // mathhelpers.cpp:184-196
    int dVert = dim + 1;
    for (int j = 0; j < dim; j++) {
        bary[j] = 0;
        for (int i = 0; i < dVert; i++) bary[j] += E[dim * i + j];
        bary[j] = bary[j] / static_cast<double>(dVert);
    }
}

void toPhys3(const double *E, const double *p, double *x) {                // mathhelpers.cpp:210-215
    for (int i = 0; i < 2; i++)
        x[i] = (E[2 + i] - E[i]) * p[0] + (E[4 + i] - E[i]) * p[1] + E[i];
}
void toPhys(const double *E, const double *p, int dim, double *x) {        // mathhelpers.cpp:217-225
    for (int i = 0; i < dim; i++) {
        x[i] = 0;
        for (int j = 0; j < dim; j++) x[i] += p[j] * (E[dim * (j + 1) + i] - E[i]);
        x[i] += E[i];
    }
}
int toRef(const double *E, const double *x, double *p) {                   // mathhelpers.cpp:227-240
    double M[4], b[2];
    M[0] = E[2] - E[0];
    M[1] = E[4] - E[0];
    M[2] = E[3] - E[1];
    M[3] = E[5] - E[1];
    b[0] = x[0] - E[0];
    b[1] = x[1] - E[1];
    return solve2x2(M, b, p);
}

void basis(const double *p, int dim, double *psi) {                        // MeshTypes.cpp:16-24
    psi[0] = 1;
    for (int i = 0; i < dim; i++) {
        psi[0] -= p[i];
        psi[i + 1] = p[i];
    }
}

// ---------------------------------------------------------------- model (model.cpp)
// k(x, labelx, y, labely). Where the reference aborts (labeled, model.cpp:74-78, 86-88) the value
// is NaN.
double kernel_value(const Mesh &m, const double *x, long lx, const double *y, long ly) {
    switch (m.kernel) {
    case K_LABELED: {  // model.cpp:67-89
        const long label = 10 * lx + ly;
        const double dist = vec_sqL2dist(x, y, 2);
        if (dist >= m.sqdelta) return NAN;
        if (label <= 12) return 0.01 * 3. / (4 * pow(m.sqdelta, 2));
        if (label >= 21) return (100 * 3. / (4 * pow(m.sqdelta, 2))) * (1 - (dist / m.sqdelta));
        if (label == 13) return 0.0;
        return NAN;
    }
    case K_NOTCH: {    // model.cpp:91-102
        const bool xN = x[1] > 0, yN = y[1] > 0, xE = x[0] > 0, yE = y[0] > 0;
        const bool cross = (xN != yN) && xE && yE;
        return !cross * (4 / (M_PI * pow(m.sqdelta, 2)));
    }
    case K_LINPROTO: {    // model.cpp:116-124
        double z[2] = {x[0] - y[0], x[1] - y[1]};
        const double denominator = 1.0 / sqrt(vec_dot(z, z, 2));
        const double c = 3.0 / (M_PI * pow(m.delta, 3));
        return c * denominator;
    }
    case K_LABELEDNOTCH:  // model.cpp:104-108
        return !(lx + ly == 7) * (4 / (M_PI * pow(m.sqdelta, 2)));
    case K_CONSTLINF:     // model.cpp:30-33
        return 3 / (4 * pow(m.sqdelta, 2));
    case K_LABELEDVALVE:  // model.cpp:110-114
        return lx >= ly ? 4.0 / (M_PI * pow(m.sqdelta, 2)) : 0.0;
    case K_CONSTTRUNC: {  // model.cpp:33-42
        double z[2] = {x[0] - y[0], x[1] - y[1]};
        const bool interacts = m.sqdelta > vec_dot(z, z, 2);
        return interacts * 4 / (M_PI * pow(m.sqdelta, 2));
    }
    case K_CONSTANT:   // model.cpp:25-28
        return 4 / (M_PI * sq(m.sqdelta));
    case K_PARABOLA: { // model.cpp:52-60
        double z[2] = {x[0] - y[0], x[1] - y[1]};
        const double value = m.sqdelta - vec_dot(z, z, 2);
        const double c = 12. / (M_PI * pow(m.sqdelta, 3));
        return c * value;
    }
    case K_FRACTIONAL: { // model.cpp:126-138
        const double exponent = m.dim + 2. * m.frac_s;
        const double constant_exponent = 2. - 2. * m.frac_s;
        double z[3];
        for (int i = 0; i < m.dim; i++) z[i] = x[i] - y[i];
        const double denominator = 1.0 / pow(sqrt(vec_dot(z, z, m.dim)), exponent);
        const double c = (constant_exponent) / (M_PI * pow(m.delta, constant_exponent));
        return c * denominator;
    }
    case K_CONSTANT3D: // model.cpp:62-65
        return 15 / (M_PI * 4 * pow(m.delta, 5));
    }
    return NAN;
}

double load_value(const Mesh &m, const double *x) {
    switch (m.load) {
    case F_LINEAR: return -2. * (x[1] + 1.);     // model.cpp:240-242
    case F_LINEAR3D: return -2. * (x[1] + 2.);   // model.cpp:259-261
    case F_CONSTANT: return 1.0;                 // model.cpp:201-203
    case F_GAUSSIAN: {                           // model.cpp:243-246
        const double sqx0 = pow(x[0], 2), sqx1 = pow(x[1], 2);
        return -4. * (sqx0 + sqx1 - 1.) * exp(-sqx0 - sqx1);
    }
    case F_JUMP: {                               // model.cpp:247-252
        const bool sign = (x[0] + x[1] - 0.5 > -EPSILON);
        return sign ? -4. : 4.;
    }
    case F_TENSORSIN:                            // model.cpp:253-255
        return 32. * pow(M_PI, 2) * sin(x[0] * M_PI * 4) * sin(x[1] * M_PI * 4);
    }
    return NAN;
}

// Forcing with outdim components (model.cpp:204-239): fo[0 .. outdim-1].
void load_vec(const Mesh &m, const double *x, double *fo) {
    const double c = M_PI / 2.0;
    switch (m.load) {
    case F_FIELD_LINEAR:                         // model.cpp:204-210
        fo[0] = -c * (1.0 + 2 * x[0]);
        fo[1] = -c * x[1];
        return;
    case F_FIELD_LINEAR3D:                       // model.cpp:211-218
        fo[0] = -c * (1.0 + 2 * x[0]) * x[1] * x[1];
        fo[1] = -c * x[1] * x[1];
        fo[2] = -c * x[2] * x[1] * x[1];
        return;
    case F_FIELD_RIGHT: fo[0] = 1.0e-1; fo[1] = 0.0; return;           // model.cpp:219-222
    case F_FIELD_DOWN: fo[0] = 0; fo[1] = -M_PI * 2; return;          // model.cpp:223-229
    case F_FIELD_BOTH: fo[0] = -M_PI; fo[1] = -M_PI * 2; return;      // model.cpp:230-239
    }
    fo[0] = load_value(m, x);
}

// Kernel with outdim x outdim components, row-major (model.cpp:140-191); scalar kernels fill kv[0].
void kernel_vec(const Mesh &m, const double *x, long lx, const double *y, long ly, double *kv) {
    switch (m.kernel) {
    case K_FIELD_CONST: {                        // model.cpp:180-191
        const double c = 4. / (M_PI * pow(m.sqdelta, 2));
        kv[0] = c; kv[1] = 0.0; kv[2] = c; kv[3] = 0.0;
        return;
    }
    case K_FIELD_PROTO: {                        // model.cpp:140-153
        double z[2] = {x[0] - y[0], x[1] - y[1]};
        const double denominator = 1.0 / pow(sqrt(vec_dot(z, z, 2)), 3);
        const double c = 3.0 / pow(m.delta, 3);
        kv[0] = c * denominator * z[0] * z[0];
        kv[1] = c * denominator * z[0] * z[1];
        kv[2] = c * denominator * z[1] * z[0];
        kv[3] = c * denominator * z[1] * z[1];
        return;
    }
    case K_FIELD_PROTO3D: {                      // model.cpp:155-178
        double z[3] = {x[0] - y[0], x[1] - y[1], x[2] - y[2]};
        const double denominator = 1.0 / pow(sqrt(vec_dot(z, z, 3)), 3);
        const double c = 3.0 / pow(m.delta, 3);
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++) kv[3 * i + j] = c * denominator * z[i] * z[j];
        return;
    }
    }
    kv[0] = kernel_value(m, x, lx, y, ly);
}

// ---------------------------------------------------------------- elements (MeshTypes.cpp:216-250)
void initializeElement(long Tdx, const Mesh &m, Elem &T) {
    for (int k = 0; k < m.dV; k++) {
        long Vdx = m.T[m.dV * Tdx + k];
        for (int j = 0; j < m.dim; j++) T.E[m.dim * k + j] = m.V[m.dim * Vdx + j];
    }
    T.absDet = absDetDim(T.E, m.dim);
    T.label = m.labT[Tdx];
    T.Tdx = Tdx;
}

// ---------------------------------------------------------------- ball truncation (integration.cpp)
bool inTriangle(const double *y, const double *p, const double *q, const double *r,
                const double *na, const double *nb, const double *nc) {   // integration.cpp:1283-1298
    double v[2];
    v[0] = y[0] - p[0]; v[1] = y[1] - p[1];
    bool a = vec_dot(na, v, 2) >= 0;
    v[0] = y[0] - q[0]; v[1] = y[1] - q[1];
    bool b = vec_dot(nb, v, 2) >= 0;
    v[0] = y[0] - r[0]; v[1] = y[1] - r[1];
    bool c = vec_dot(nc, v, 2) >= 0;
    return a && b && c;
}

int placePointOnCap(const double *ypred, const double *ycur, const double *x, double sqdelta,
                    const double *TE, const double *na, const double *nb, const double *nc,
                    double orientation, int Rdx, double *R) {             // integration.cpp:1353-1377
    double n[2], ynew[2];
    rightNormal(ycur, ypred, orientation, n);
    double s = sqrt(sqdelta / vec_dot(n, n, 2));
    n[0] = n[0] * s;
    n[1] = n[1] * s;
    ynew[0] = x[0] + n[0];
    ynew[1] = x[1] + n[1];
    if (inTriangle(ynew, &TE[0], &TE[2], &TE[4], na, nb, nc)) {
        if (Rdx >= 9) return 0;   // see method_retriangulate: R holds 9 points
        R[2 * Rdx] = ynew[0];
        R[2 * Rdx + 1] = ynew[1];
        return 1;
    }
    return 0;
}

// The reference's point buffer R holds 9 points (integration.cpp:1415). Where the sphere touches
// an edge up to rounding (on an unjittered grid with h = 0.15 and delta = 0.1, element centroids
// lie at distance delta from grid lines), that edge yields two
// roots about 1e-8 apart with a cap point between them; with two such edges the polygon has 10
// or more points and the reference writes past R (undefined behaviour). Here, as in the CUDA
// restatement, points beyond the 9th are dropped.
int method_retriangulate(const double *xc, const double *TE, double sqdelta, double *out,
                         int caps) {                                       // integration.cpp:1393-1512
    int Rdx = 0;
    double na[2], nb[2], nc[2];
    bool is_onEdge = false, is_firstPointLiesOnVertex = true;
    double R[9 * 2];
    for (int i = 0; i < 18; i++) R[i] = 0;
    double orientation = -signDet2(TE);
    rightNormal(&TE[0], &TE[2], orientation, na);
    rightNormal(&TE[2], &TE[4], orientation, nb);
    rightNormal(&TE[4], &TE[0], orientation, nc);
    for (int k = 0; k < 3; k++) {
        const double *p = &TE[2 * k];
        const double *q = &TE[2 * ((k + 1) % 3)];
        double a[2] = {q[0] - xc[0], q[1] - xc[1]};
        double b[2] = {p[0] - q[0], p[1] - q[1]};
        if (vec_sqL2dist(p, xc, 2) <= sqdelta) {
            if (Rdx < 9) {
                R[2 * Rdx] = p[0];
                R[2 * Rdx + 1] = p[1];
                Rdx += 1;
            }
            is_onEdge = false;
        }
        // arma::dot of two 2-vectors: a0*b0 + a1*b1
        double ab = a[0] * b[0] + a[1] * b[1];
        double aa = a[0] * a[0] + a[1] * a[1];
        double bb = b[0] * b[0] + b[1] * b[1];
        double v = sq(ab) - (aa - sqdelta) * bb;
        if (v >= 0) {
            double term1 = -ab / bb;
            double term2 = sqrt(v) / bb;
            double lam1, lam2;
            if (term1 > 0) {
                lam1 = term1 + term2;
                lam2 = 1 / lam1 * (aa - sqdelta) / bb;
            } else {
                lam2 = term1 - term2;
                lam1 = 1 / lam2 * (aa - sqdelta) / bb;
            }
            double y1[2] = {lam1 * b[0] + q[0], lam1 * b[1] + q[1]};
            double y2[2] = {lam2 * b[0] + q[0], lam2 * b[1] + q[1]};
            if ((0 <= lam1) && (lam1 <= 1)) {
                is_firstPointLiesOnVertex = is_firstPointLiesOnVertex && (bool)Rdx;
                if (is_onEdge && caps)
                    Rdx += placePointOnCap(&R[2 * (Rdx - 1)], y1, xc, sqdelta, TE, na, nb, nc, orientation, Rdx, R);
                if (Rdx < 9) {
                    R[2 * Rdx] = y1[0];
                    R[2 * Rdx + 1] = y1[1];
                    Rdx += 1;
                }
                is_onEdge = true;
            }
            if ((0 <= lam2) && (lam2 <= 1) && (sq(lam1 - lam2) > 0)) {
                is_firstPointLiesOnVertex = is_firstPointLiesOnVertex && (bool)Rdx;
                if (is_onEdge && caps)
                    Rdx += placePointOnCap(&R[2 * (Rdx - 1)], y2, xc, sqdelta, TE, na, nb, nc, orientation, Rdx, R);
                if (Rdx < 9) {
                    R[2 * Rdx] = y2[0];
                    R[2 * Rdx + 1] = y2[1];
                    Rdx += 1;
                }
                is_onEdge = true;
            }
        }
    }
    if (is_onEdge && (!is_firstPointLiesOnVertex && Rdx > 1) && caps)
        Rdx += placePointOnCap(&R[2 * (Rdx - 1)], &R[0], xc, sqdelta, TE, na, nb, nc, orientation, Rdx, R);
    if (Rdx < 3) return 0;
    for (int k = 0; k < Rdx - 2; k++) {
        for (int i = 0; i < 2; i++) {
            out[2 * (3 * k + 0) + i] = R[i];
            out[2 * (3 * k + 1) + i] = R[2 * (k + 1) + i];
            out[2 * (3 * k + 2) + i] = R[2 * (k + 2) + i];
        }
    }
    return Rdx - 2;
}

// placePointCapCenter (integration.cpp:1300-1351): the circular segment of B_delta(x) cut off by
// the chord y_pred - y_cur. Its centroid lies on the chord's outward normal at distance
// 4 delta sin^3(alpha) / (3 (2 alpha - sin 2 alpha)) from x (alpha: half the opening angle); if
// it lies in the triangle it is written to cap and the segment's area (delta^2 / 2)
// (2 alpha - sin 2 alpha) is returned, else 0.
double placePointCapCenter(const double *ypred, const double *ycur, const double *xc, double sqdelta,
                           const double *TE, const double *na, const double *nb, const double *nc,
                           double orientation, double *cap) {
    double p1[2] = {xc[0] + ypred[0] * -1, xc[1] + ypred[1] * -1};
    double p2[2] = {xc[0] + ycur[0] * -1, xc[1] + ycur[1] * -1};
    const double alpha = 0.5 * acos(vec_dot(p1, p2, 2) / sqdelta);
    double s[2];
    rightNormal(ycur, ypred, orientation, s);
    const double scalingFactor = (4 * sqrt(sqdelta) * pow(sin(alpha), 3)) / (3 * (2 * alpha - sin(2 * alpha))) *
                                 sqrt(1. / vec_dot(s, s, 2));
    double centroid[2] = {xc[0] + s[0] * scalingFactor, xc[1] + s[1] * scalingFactor};
    if (inTriangle(centroid, &TE[0], &TE[2], &TE[4], na, nb, nc)) {
        cap[0] = centroid[0];
        cap[1] = centroid[1];
        return (sqdelta / 2) * (2 * alpha - sin(2 * alpha));
    }
    return 0.0;
}

// method_exact (integration.cpp:1632-1761): the polygon of B_delta(x) and T without cap points
// (fan sub-triangles in out, their number returned), and up to three circular segments (caps,
// weights, *nCaps). Points beyond R's 9 are dropped, as in method_retriangulate.
int method_exact(const double *xc, const double *TE, double sqdelta, double *out, double *caps,
                 double *capw, int *nCaps) {
    *nCaps = 0;
    int Rdx = 0;
    double na[2], nb[2], nc[2];
    bool is_onEdge = false, is_firstPointLiesOnVertex = true;
    double R[9 * 2];
    for (int i = 0; i < 18; i++) R[i] = 0;
    const double orientation = -signDet2(TE);
    rightNormal(&TE[0], &TE[2], orientation, na);
    rightNormal(&TE[2], &TE[4], orientation, nb);
    rightNormal(&TE[4], &TE[0], orientation, nc);
    for (int k = 0; k < 3; k++) {
        const double *p = &TE[2 * k];
        const double *q = &TE[2 * ((k + 1) % 3)];
        double a[2] = {q[0] - xc[0], q[1] - xc[1]};
        double b[2] = {p[0] - q[0], p[1] - q[1]};
        if (vec_sqL2dist(p, xc, 2) <= sqdelta) {
            if (Rdx < 9) { R[2 * Rdx] = p[0]; R[2 * Rdx + 1] = p[1]; Rdx += 1; }
            is_onEdge = false;
        }
        const double ab = a[0] * b[0] + a[1] * b[1];
        const double aa = a[0] * a[0] + a[1] * a[1];
        const double bb = b[0] * b[0] + b[1] * b[1];
        const double v = sq(ab) - (aa - sqdelta) * bb;
        if (v >= 0) {
            const double term1 = -ab / bb;
            const double term2 = sqrt(v) / bb;
            double lam1, lam2;
            if (term1 > 0) {
                lam1 = term1 + term2;
                lam2 = 1 / lam1 * (aa - sqdelta) / bb;
            } else {
                lam2 = term1 - term2;
                lam1 = 1 / lam2 * (aa - sqdelta) / bb;
            }
            const double y1[2] = {lam1 * b[0] + q[0], lam1 * b[1] + q[1]};
            const double y2[2] = {lam2 * b[0] + q[0], lam2 * b[1] + q[1]};
            if ((0 <= lam1) && (lam1 <= 1)) {
                is_firstPointLiesOnVertex = is_firstPointLiesOnVertex && (bool)Rdx;
                if (is_onEdge && *nCaps < 3) {
                    capw[*nCaps] = placePointCapCenter(&R[2 * (Rdx - 1)], y1, xc, sqdelta, TE, na, nb, nc, orientation, &caps[2 * *nCaps]);
                    *nCaps += !double_eq(capw[*nCaps], 0.);
                }
                if (Rdx < 9) { R[2 * Rdx] = y1[0]; R[2 * Rdx + 1] = y1[1]; Rdx += 1; }
                is_onEdge = true;
            }
            if ((0 <= lam2) && (lam2 <= 1) && (sq(lam1 - lam2) > 0)) {
                is_firstPointLiesOnVertex = is_firstPointLiesOnVertex && (bool)Rdx;
                if (is_onEdge && *nCaps < 3) {
                    capw[*nCaps] = placePointCapCenter(&R[2 * (Rdx - 1)], y2, xc, sqdelta, TE, na, nb, nc, orientation, &caps[2 * *nCaps]);
                    *nCaps += !double_eq(capw[*nCaps], 0.);
                }
                if (Rdx < 9) { R[2 * Rdx] = y2[0]; R[2 * Rdx + 1] = y2[1]; Rdx += 1; }
                is_onEdge = true;
            }
        }
    }
    if (is_onEdge && *nCaps < 3) {
        capw[*nCaps] = placePointCapCenter(&R[2 * (Rdx - 1)], &R[0], xc, sqdelta, TE, na, nb, nc, orientation, &caps[2 * *nCaps]);
        *nCaps += !double_eq(capw[*nCaps], 0.);
    }
    if (Rdx < 3) return 0;
    for (int k = 0; k < Rdx - 2; k++)
        for (int i = 0; i < 2; i++) {
            out[2 * (3 * k + 0) + i] = R[i];
            out[2 * (3 * k + 1) + i] = R[2 * (k + 1) + i];
            out[2 * (3 * k + 2) + i] = R[2 * (k + 2) + i];
        }
    return Rdx - 2;
}

int method_baryCenter(const double *x, const Elem &T, const Mesh &m) {    // integration.cpp:1262-1280
    double b[3];
    baryCenter(m.dim, T.E, b);
    double distance = vec_sqL2dist(x, b, m.dim);
    return (distance > m.sqdelta) ? 0 : -1;
}

// ---------------------------------------------------------------- integration routines
// method_retriangulateInfty (integration.cpp:1521-1623): B_inf(x) (the square of half side delta)
// intersected with T. Its points are T's vertices inside the square, the edges' crossings of the
// square's sides, and the square's corners inside T. The reference inserts them into a
// CGAL::Triangulation_2 (CGAL, not in this tree), which triangulates their convex hull. Here the
// hull (Andrew's monotone chain, exact duplicates and collinear points dropped) is fanned from its
// first point. Both cover the same convex polygon, so the rules integrate polynomial integrands
// (the constantLinf2D kernel times the P1 basis) alike up to rounding; the sub-triangles differ.
static double vec_LInfdist(const double *x, const double *y, int len) {   // mathhelpers.cpp:281-288
    double r = 0;
    for (int i = 0; i < len; i++) r = std::max(absolute(x[i] - y[i]), r);
    return r;
}

int method_retriangulateInfty(const double *xc, const double *TE, double sqdelta, double *out) {
    const double delta = sqrt(sqdelta);
    std::vector<std::pair<double, double>> pts;
    for (int k = 0; k < 3; k++) {
        const double *p = &TE[2 * k];
        const double *q = &TE[2 * ((k + 1) % 3)];
        if (vec_LInfdist(p, xc, 2) <= delta) pts.emplace_back(p[0], p[1]);
        const double b[2] = {p[0] - q[0], p[1] - q[1]};
        double lambda[4] = {0, 0, 0, 0};
        if (absolute(b[0]) > 0.) {
            lambda[0] = (xc[0] + delta - q[0]) / b[0];
            lambda[1] = (xc[0] - delta - q[0]) / b[0];
        }
        if (absolute(b[1]) > 0.) {
            lambda[2] = (xc[1] + delta - q[1]) / b[1];
            lambda[3] = (xc[1] - delta - q[1]) / b[1];
        }
        for (double l : lambda) {
            if ((l > 0.) && (l < 1.)) {
                const double xp[2] = {q[0] + b[0] * l, q[1] + b[1] * l};
                if (vec_LInfdist(xp, xc, 2) <= delta * (1 + EPSILON)) pts.emplace_back(xp[0], xp[1]);
            }
        }
    }
    double na[2], nb[2], nc[2];
    const double orientation = -signDet2(TE);
    rightNormal(&TE[0], &TE[2], orientation, na);
    rightNormal(&TE[2], &TE[4], orientation, nb);
    rightNormal(&TE[4], &TE[0], orientation, nc);
    const double sx[4] = {1, 1, -1, -1}, sy[4] = {1, -1, -1, 1};
    for (int c = 0; c < 4; c++) {
        const double v[2] = {xc[0] + sx[c] * delta, xc[1] + sy[c] * delta};
        if (inTriangle(v, &TE[0], &TE[2], &TE[4], na, nb, nc)) pts.emplace_back(v[0], v[1]);
    }
    std::sort(pts.begin(), pts.end());
    pts.erase(std::unique(pts.begin(), pts.end()), pts.end());
    if (pts.size() < 3) return 0;
    auto cross = [](const std::pair<double, double> &o, const std::pair<double, double> &a,
                    const std::pair<double, double> &b) {
        return (a.first - o.first) * (b.second - o.second) - (a.second - o.second) * (b.first - o.first);
    };
    std::vector<std::pair<double, double>> h(2 * pts.size());
    size_t n = 0;
    for (size_t i = 0; i < pts.size(); i++) {   // lower hull
        while (n >= 2 && cross(h[n - 2], h[n - 1], pts[i]) <= 0) n--;
        h[n++] = pts[i];
    }
    for (size_t i = pts.size() - 1, t = n + 1; i-- > 0;) {   // upper hull
        while (n >= t && cross(h[n - 2], h[n - 1], pts[i]) <= 0) n--;
        h[n++] = pts[i];
    }
    n--;   // the last point repeats the first
    if (n < 3) return 0;
    for (size_t k = 0; k + 2 < n; k++) {
        const std::pair<double, double> t3[3] = {h[0], h[k + 1], h[k + 2]};
        for (int j = 0; j < 3; j++) {
            out[2 * (3 * k + j) + 0] = t3[j].first;
            out[2 * (3 * k + j) + 1] = t3[j].second;
        }
    }
    return (int)n - 2;
}

// The retriangulation of the configured ball (Cassemble.cpp:134-141): L2 or L-infinity.
int retri_method(const Mesh &m, const double *x, const double *TE, double *out) {
    return m.linf ? method_retriangulateInfty(x, TE, m.sqdelta, out) : method_retriangulate(x, TE, m.sqdelta, out, m.caps);
}

// All four local blocks are (dV x dV) row-major, outdim = 1.
int integrate_retriangulate(const Elem &aT, const Elem &bT, const Quad &q, const Mesh &m,
                            double *tL, double *tN, double *tLP, double *tNP) {  // integration.cpp:345-540
    const int dV = 3;
    double x[2], y[2], ref[2], psi[3];
    double innerLocal, innerNonloc[3], innerNonlocPrime[3];
    double reTri[9 * 3 * 2];
    int doesInteract = 0;
    for (int k = 0; k < q.nPx; k++) {
        toPhys(aT.E, &q.Px[2 * k], 2, x);
        int Rdx = retri_method(m, x, bT.E, reTri);
        doesInteract += Rdx;
        innerLocal = 0;
        for (int b = 0; b < dV; b++) { innerNonloc[b] = 0; innerNonlocPrime[b] = 0; }
        for (int r = 0; r < Rdx; r++) {
            for (int i = 0; i < q.nPy; i++) {
                toPhys3(&reTri[6 * r], &q.Py[2 * i], y);
                double rTdet = absDet2(&reTri[6 * r]);
                double ker = kernel_value(m, x, aT.label, y, bT.label);
                innerLocal += ker * q.dy[i] * rTdet;
                toRef(bT.E, y, ref);
                double kerP = kernel_value(m, y, bT.label, x, aT.label);
                basis(ref, 2, psi);
                for (int b = 0; b < dV; b++) {
                    innerNonloc[b] += psi[b] * ker * q.dy[i] * rTdet;
                    innerNonlocPrime[b] += psi[b] * kerP * q.dy[i] * rTdet;
                }
                for (int a = 0; a < dV; a++)
                    for (int b = 0; b < dV; b++)
                        tLP[dV * a + b] += psi[a] * psi[b] * kerP * q.dy[i] * q.dx[k] * rTdet * aT.absDet;
            }
        }
        for (int a = 0; a < dV; a++) {
            for (int b = 0; b < dV; b++) {
                tL[dV * a + b] += aT.absDet * q.psix[dV * k + a] * q.psix[dV * k + b] * q.dx[k] * innerLocal;
                tN[dV * a + b] += aT.absDet * q.psix[dV * k + a] * q.dx[k] * innerNonloc[b];
                tNP[dV * a + b] += aT.absDet * q.psix[dV * k + a] * q.dx[k] * innerNonlocPrime[b];
            }
        }
    }
    return (doesInteract || m.full_search);
}

// integrate_exact, "exactBall" (integration.cpp:706-907): the polygon of method_exact with the
// inner rule and each circular segment with one point at its centroid weighted by its exact
// area; weight 2, termNonloc with k(y, x).
int integrate_exact(const Elem &aT, const Elem &bT, const Quad &q, const Mesh &m, double *tL, double *tN) {
    const int dV = 3;
    double x[2], y[2], ref[2], psi[3];
    double reTri[9 * 3 * 2], caps[6] = {0, 0, 0, 0, 0, 0}, capw[3] = {0, 0, 0};
    int nCaps = 0, doesInteract = 0;
    for (int k = 0; k < q.nPx; k++) {
        toPhys(aT.E, &q.Px[2 * k], 2, x);
        const int Rdx = method_exact(x, bT.E, m.sqdelta, reTri, caps, capw, &nCaps);
        doesInteract += Rdx;
        double innerLocal = 0, innerNonloc[3] = {0, 0, 0};
        for (int r = 0; r < Rdx; r++) {
            for (int i = 0; i < q.nPy; i++) {
                toPhys3(&reTri[6 * r], &q.Py[2 * i], y);
                const double rTdet = absDet2(&reTri[6 * r]);
                double ker = kernel_value(m, x, aT.label, y, bT.label);
                innerLocal += ker * q.dy[i] * rTdet;
                toRef(bT.E, y, ref);
                ker = kernel_value(m, y, bT.label, x, aT.label);
                basis(ref, 2, psi);
                for (int b = 0; b < dV; b++) innerNonloc[b] += psi[b] * ker * q.dy[i] * rTdet;
            }
        }
        for (int i = 0; i < nCaps; i++) {
            double ker = kernel_value(m, x, aT.label, &caps[2 * i], bT.label);
            innerLocal += ker * capw[i];
            toRef(bT.E, &caps[2 * i], ref);
            ker = kernel_value(m, &caps[2 * i], bT.label, x, aT.label);
            basis(ref, 2, psi);
            for (int b = 0; b < dV; b++) innerNonloc[b] += psi[b] * ker * capw[i];
        }
        for (int a = 0; a < dV; a++)
            for (int b = 0; b < dV; b++) {
                tL[dV * a + b] += 2 * aT.absDet * q.psix[dV * k + a] * q.psix[dV * k + b] * q.dx[k] * innerLocal;
                tN[dV * a + b] += 2 * aT.absDet * q.psix[dV * k + a] * q.dx[k] * innerNonloc[b];
            }
    }
    return (doesInteract || m.full_search);
}

int integrate_baryCenter(const Elem &aT, const Elem &bT, const Quad &q, const Mesh &m,
                         double *tL, double *tN) {                        // integration.cpp:910-1018
    const int dim = m.dim, dV = m.dV;
    double x[3], y[3];
    double innerLocal, innerNonloc[4];
    int doesInteract = 0;
    for (int k = 0; k < q.nPx; k++) {
        toPhys(aT.E, &q.Px[dim * k], dim, x);
        innerLocal = 0;
        for (int b = 0; b < dV; b++) innerNonloc[b] = 0;
        int Rdx = method_baryCenter(x, bT, m);
        doesInteract += Rdx;
        if (Rdx) {
            for (int i = 0; i < q.nPy; i++) {
                toPhys(bT.E, &q.Py[dim * i], dim, y);
                double rTdet = absDetDim(bT.E, dim);
                double ker = kernel_value(m, x, aT.label, y, bT.label);
                innerLocal += rTdet * ker * q.dy[i];
                ker = kernel_value(m, y, bT.label, x, aT.label);
                for (int b = 0; b < dV; b++) innerNonloc[b] += q.psiy[dV * i + b] * ker * q.dy[i] * rTdet;
            }
        }
        for (int a = 0; a < dV; a++) {
            for (int b = 0; b < dV; b++) {
                tL[dV * a + b] += 2 * aT.absDet * q.psix[dV * k + a] * q.psix[dV * k + b] * q.dx[k] * innerLocal;
                tN[dV * a + b] += 2 * aT.absDet * q.psix[dV * k + a] * q.dx[k] * innerNonloc[b];
            }
        }
    }
    return (doesInteract || m.full_search);
}

// integrate_retriangulate_unysmm (integration.cpp:542-704): the retriangulated inner domain with
// weight 2; termNonloc takes k(y, x); no prime blocks.
int integrate_retriangulate_unsymm(const Elem &aT, const Elem &bT, const Quad &q, const Mesh &m,
                                   double *tL, double *tN) {
    const int dV = 3;
    double x[2], y[2], ref[2], psi[3];
    double reTri[9 * 3 * 2];
    int doesInteract = 0;
    for (int k = 0; k < q.nPx; k++) {
        toPhys(aT.E, &q.Px[2 * k], 2, x);
        const int Rdx = retri_method(m, x, bT.E, reTri);
        doesInteract += Rdx;
        double innerLocal = 0, innerNonloc[3] = {0, 0, 0};
        for (int r = 0; r < Rdx; r++) {
            for (int i = 0; i < q.nPy; i++) {
                toPhys3(&reTri[6 * r], &q.Py[2 * i], y);
                const double rTdet = absDet2(&reTri[6 * r]);
                double ker = kernel_value(m, x, aT.label, y, bT.label);
                innerLocal += ker * q.dy[i] * rTdet;
                toRef(bT.E, y, ref);
                ker = kernel_value(m, y, bT.label, x, aT.label);
                basis(ref, 2, psi);
                for (int b = 0; b < dV; b++) innerNonloc[b] += psi[b] * ker * q.dy[i] * rTdet;
            }
        }
        for (int a = 0; a < dV; a++)
            for (int b = 0; b < dV; b++) {
                tL[dV * a + b] += 2 * aT.absDet * q.psix[dV * k + a] * q.psix[dV * k + b] * q.dx[k] * innerLocal;
                tN[dV * a + b] += 2 * aT.absDet * q.psix[dV * k + a] * q.dx[k] * innerNonloc[b];
            }
    }
    return (doesInteract || m.full_search);
}

// method_subSuperSetBalls (integration.cpp:1251-1260): vertices of T strictly inside the ball.
int method_subSuperSetBalls(const double *x, const Elem &T, const Mesh &m) {
    int n = 0;
    for (int i = 0; i < m.dV; i++) n += (vec_sqL2dist(x, &T.E[m.dim * i], m.dim) < m.sqdelta);
    return n;
}

// integrate_subSuperSetBalls (integration.cpp:1021-1095): the whole inner element, weighted by
// averageWeights[#vertices inside - 1] (subSetBall: (0, 0, 1); averageBall: (0.5, 0.5, 1)).
int integrate_subSuperSetBalls(const Elem &aT, const Elem &bT, const Quad &q, const Mesh &m, int method,
                               double *tL, double *tN) {
    const int dim = m.dim, dV = m.dV;
    double W[4] = {0, 0, 0, 0};
    if (method == M_AVERAGE) for (int i = 0; i < dV; i++) W[i] = 0.5;
    W[2] = 1.0;
    double x[3], y[3];
    int doesInteract = 0;
    for (int k = 0; k < q.nPx; k++) {
        toPhys(aT.E, &q.Px[dim * k], dim, x);
        double innerLocal = 0, innerNonloc[4] = {0, 0, 0, 0};
        const int nContained = method_subSuperSetBalls(x, bT, m);
        doesInteract += nContained;
        if (nContained >= 1) {
            for (int i = 0; i < q.nPy; i++) {
                toPhys(bT.E, &q.Py[dim * i], dim, y);
                const double rTdet = absDetDim(bT.E, dim);
                double ker = kernel_value(m, x, aT.label, y, bT.label);
                innerLocal += W[nContained - 1] * rTdet * ker * q.dy[i];
                ker = kernel_value(m, y, bT.label, x, aT.label);
                for (int b = 0; b < dV; b++)
                    innerNonloc[b] += W[nContained - 1] * q.psiy[dV * i + b] * ker * q.dy[i] * rTdet;
            }
        }
        for (int a = 0; a < dV; a++)
            for (int b = 0; b < dV; b++) {
                tL[dV * a + b] += 2 * aT.absDet * q.psix[dV * k + a] * q.psix[dV * k + b] * q.dx[k] * innerLocal;
                tN[dV * a + b] += 2 * aT.absDet * q.psix[dV * k + a] * q.dx[k] * innerNonloc[b];
            }
    }
    return (doesInteract || m.full_search);
}

// integrate_baryCenterRT (integration.cpp:1155-1249): the outer domain is the part of aT inside the
// ball around bT's barycenter (retriangulated), the inner element is whole, weight 2. The
// reference reads innerNonloc[outdim * (a % outdim) + b % outdim], which is innerNonloc[0] for
// every (a, b) at outdim 1; kept as is.
int integrate_baryCenterRT(const Elem &aT, const Elem &bT, const Quad &q, const Mesh &m,
                           double *tL, double *tN) {
    const int dV = 3;
    double bc[2], xq[2], y[2], ref[2], psix[3];
    double reTri[9 * 3 * 2];
    baryCenter(2, bT.E, bc);
    const int Rdx = method_retriangulate(bc, aT.E, m.sqdelta, reTri, m.caps);
    if (!Rdx) return m.full_search;
    const double bTdet = absDet2(bT.E);
    for (int r = 0; r < Rdx; r++) {
        const double rTdet = absDet2(&reTri[6 * r]);
        for (int k = 0; k < q.nPx; k++) {
            toPhys(&reTri[6 * r], &q.Px[2 * k], 2, xq);
            double innerLocal = 0, innerNonloc[3] = {0, 0, 0};
            for (int i = 0; i < q.nPy; i++) {
                toPhys(bT.E, &q.Py[2 * i], 2, y);
                double ker = kernel_value(m, xq, aT.label, y, bT.label);
                innerLocal += ker * q.dy[i] * bTdet;
                ker = kernel_value(m, y, bT.label, xq, aT.label);
                for (int b = 0; b < dV; b++) innerNonloc[b] += q.psiy[dV * i + b] * ker * q.dy[i] * bTdet;
            }
            toRef(aT.E, xq, ref);
            basis(ref, 2, psix);
            for (int a = 0; a < dV; a++)
                for (int b = 0; b < dV; b++) {
                    tL[dV * a + b] += 2 * rTdet * psix[a] * psix[b] * q.dx[k] * innerLocal;
                    tN[dV * a + b] += 2 * rTdet * psix[a] * q.dx[k] * innerNonloc[0];
                }
        }
    }
    return 1;
}

// integrate_fullyContained (integration.cpp:290-343), "noTruncation": both whole elements, all
// four blocks; every pair interacts.
int integrate_fullyContained(const Elem &aT, const Elem &bT, const Quad &q, const Mesh &m,
                             double *tL, double *tN, double *tLP, double *tNP) {
    const int dim = m.dim, dV = m.dV;
    double x[3], y[3];
    for (int k = 0; k < q.nPx; k++) {
        toPhys(aT.E, &q.Px[dim * k], dim, x);
        for (int i = 0; i < q.nPy; i++) {
            toPhys(bT.E, &q.Py[dim * i], dim, y);
            const double ker = kernel_value(m, x, aT.label, y, bT.label);
            const double kerP = kernel_value(m, y, bT.label, x, aT.label);
            for (int a = 0; a < dV; a++)
                for (int b = 0; b < dV; b++) {
                    const double f = q.dx[k] * q.dy[i] * aT.absDet * bT.absDet;
                    tL[dV * a + b] += f * q.psix[dV * k + a] * q.psix[dV * k + b] * ker;
                    tLP[dV * a + b] += f * q.psiy[dV * i + a] * q.psiy[dV * i + b] * kerP;
                    tN[dV * a + b] += f * q.psix[dV * k + a] * q.psiy[dV * i + b] * kerP;
                    tNP[dV * a + b] += f * q.psix[dV * k + a] * q.psiy[dV * i + b] * ker;
                }
        }
    }
    return 1;
}

// join + setupElement: integration.cpp:1897-1958
int join(const Elem &aT, const Elem &bT, const Mesh &m, Elem &aS, Elem &bS, int *argA, int *argB) {
    int nEqual = 0;
    int AinB[3] = {0, 0, 0}, BinA[3] = {0, 0, 0};
    const long *aV = &m.T[3 * aT.Tdx];
    const long *bV = &m.T[3 * bT.Tdx];
    long aS_v[3], bS_v[3];
    for (int a = 0; a < 3; a++) {
        for (int b = 0; b < 3; b++) {
            if (aV[a] == bV[b]) {
                AinB[a] += 1;
                BinA[b] += 1;
                aS_v[nEqual] = aV[a];
                argA[nEqual] = a;
                bS_v[nEqual] = bV[b];
                argB[nEqual] = b;
                nEqual += 1;
            }
        }
    }
    int ia = 0, ib = 0;
    for (int i = 0; i < 3; i++) {
        if (!AinB[i]) { aS_v[nEqual + ia] = aV[i]; argA[nEqual + ia] = i; ia++; }
        if (!BinA[i]) { bS_v[nEqual + ib] = bV[i]; argB[nEqual + ib] = i; ib++; }
    }
    for (int k = 0; k < 3; k++)
        for (int j = 0; j < 2; j++) {
            aS.E[2 * k + j] = m.V[2 * aS_v[k] + j];
            bS.E[2 * k + j] = m.V[2 * bS_v[k] + j];
        }
    aS.absDet = absDetDim(aS.E, 2);
    bS.absDet = absDetDim(bS.E, 2);
    return nEqual;
}

int integrate_fractional(const Elem &aT, const Elem &bT, const Quad &q, const Mesh &m,
                         double *tL, double *tN, double *tLP, double *tNP) {  // integration.cpp:187-288
    Elem aS, bS;
    int argA[3], argB[3];
    const int nEqual = join(aT, bT, m, aS, bS, argA, argB);
    if (nEqual < 1 || nEqual > 3) return -1;  // reference aborts
    const int c = nEqual - 1;
    const int nT = (nEqual == 1) ? 2 : (nEqual == 2 ? 5 : 6);
    const int dV = 3;
    const int nLocal = 2 * dV - nEqual;
    double x[2], y[2], psix[3], psiy[3], psixy[6];
    for (int t = 0; t < nT; t++) {
        for (int k = 0; k < q.nPg; k++) {
            const double tf = q.tdetFrac[c][t * q.nPg + k];
            const double *al = &q.alphaC[c][(t * q.nPg + k) * 4];
            toPhys(aS.E, &al[0], 2, x);
            toPhys(bS.E, &al[2], 2, y);
            double ker = kernel_value(m, x, aT.label, y, bT.label);
            basis(&al[0], 2, psix);
            basis(&al[2], 2, psiy);
            int shift = dV - nEqual;
            for (int a = 0; a < nEqual; a++) psixy[a] = psix[a] - psiy[a];
            for (int a = nEqual; a < dV; a++) {
                psixy[a] = psix[a];
                psixy[a + shift] = -psiy[a];
            }
            for (int a = 0; a < nLocal; a++) {
                for (int b = 0; b < nLocal; b++) {
                    double f = ker * tf * psixy[a] * psixy[b] * q.dg[k] * aS.absDet * bS.absDet;
                    if (a < dV) {
                        if (b < dV) tL[dV * argA[a] + argA[b]] += f;
                        else tN[dV * argA[a] + argB[b - shift]] -= f;
                    } else {
                        if (b < dV) tNP[dV * argA[b] + argB[a - shift]] -= f;
                        else tLP[dV * argB[a - shift] + argB[b - shift]] += f;
                    }
                }
            }
        }
    }
    return 1;
}

// integrate_weakSingular (integration.cpp:82-185): the Duffy maps of integrate_fractional with
// the kernel at the canceled points, the basis functions at the points with xi kept, and the
// determinant with xi^(1 - 2s); termNonlocPrime equals termNonloc.
int integrate_weakSingular(const Elem &aT, const Elem &bT, const Quad &q, const Mesh &m,
                           double *tL, double *tN, double *tLP, double *tNP) {
    Elem aS, bS;
    int argA[3], argB[3];
    const int nEqual = join(aT, bT, m, aS, bS, argA, argB);
    if (nEqual < 1 || nEqual > 3) return -1;  // reference aborts
    const int c = nEqual - 1;
    const int nT = (nEqual == 1) ? 2 : (nEqual == 2 ? 5 : 6);
    const int dV = 3;
    double xc[2], yc[2], psix[3], psiy[3];
    for (int t = 0; t < nT; t++) {
        for (int k = 0; k < q.nPg; k++) {
            const double tw = q.tdetWeak[c][t * q.nPg + k];
            const double *ac = &q.alphaC[c][(t * q.nPg + k) * 4];
            const double *au = &q.alphaU[c][(t * q.nPg + k) * 4];
            toPhys(aS.E, &ac[0], 2, xc);
            toPhys(bS.E, &ac[2], 2, yc);
            const double ker = kernel_value(m, xc, aT.label, yc, bT.label);
            basis(&au[0], 2, psix);
            basis(&au[2], 2, psiy);
            for (int a = 0; a < dV; a++)
                for (int b = 0; b < dV; b++) {
                    const double f = ker * tw * q.dg[k] * aS.absDet * bS.absDet;
                    tL[dV * argA[a] + argA[b]] += f * psix[a] * psix[b];
                    tLP[dV * argB[a] + argB[b]] += f * psiy[a] * psiy[b];
                    tN[dV * argA[a] + argB[b]] += f * psix[a] * psiy[b];
                    tNP[dV * argA[a] + argB[b]] += f * psix[a] * psiy[b];
                }
        }
    }
    return 1;
}

// Duffy tables: MeshTypes.cpp:32-209 (traffo*), :252-327 (initializeQuadrule), mathhelpers.cpp:88-97
double traffo(int c, int t, double *al) {
    const double xi = al[0], e1 = al[1], e2 = al[2], e3 = al[3];
    if (c == 0) {
        if (t == 0) { al[0] = xi; al[1] = e1 * xi; al[2] = e2 * xi; al[3] = e2 * e3 * xi; }
        else { al[0] = xi * e2; al[1] = xi * e2 * e3; al[2] = xi; al[3] = xi * e1; }
        return pow(xi, 3) * e2;
    }
    if (c == 1) {
        switch (t) {
        case 0:
            al[0] = xi; al[1] = xi * e1 * e3; al[2] = xi * (1. - e1 * e2); al[3] = xi * e1 * (1. - e2);
            return pow(xi, 3) * sq(e1);
        case 1:
            al[0] = xi; al[1] = xi * e1; al[2] = xi * (1. - e1 * e2 * e3); al[3] = xi * e1 * e2 * (1. - e3);
            break;
        case 2:
            al[0] = xi * (1. - e1 * e2); al[1] = xi * e1 * (1. - e2); al[2] = xi; al[3] = xi * e1 * e2 * e3;
            break;
        case 3:
            al[0] = xi * (1. - e1 * e2 * e3); al[1] = xi * e1 * e2 * (1. - e3); al[2] = xi; al[3] = xi * e1;
            break;
        default:
            al[0] = xi * (1. - e1 * e2 * e3); al[1] = xi * e1 * (1. - e2 * e3); al[2] = xi; al[3] = xi * e1 * e2;
            break;
        }
        return pow(xi, 3) * sq(e1) * e2;
    }
    switch (t) {
    case 0:
        al[0] = xi; al[1] = xi * (1. - e1 + e1 * e2); al[2] = xi * (1. - e1 * e2 * e3); al[3] = xi * (1. - e1);
        break;
    case 1:
        al[0] = xi * (1. - e1 * e2 * e3); al[1] = xi * (1. - e1); al[2] = xi; al[3] = xi * (1. - e1 + e1 * e2);
        break;
    case 2:
        al[0] = xi; al[1] = xi * e1 * (1. - e2 + e2 * e3); al[2] = xi * (1. - e1 * e2); al[3] = xi * e1 * (1. - e2);
        break;
    case 3:
        al[0] = xi * (1. - e1 * e2); al[1] = xi * e1 * (1. - e2); al[2] = xi; al[3] = xi * e1 * (1. - e2 + e2 * e3);
        break;
    case 4:
        al[0] = xi * (1. - e1 * e2 * e3); al[1] = xi * e1 * (1. - e2 * e3); al[2] = xi; al[3] = xi * e1 * (1. - e2);
        break;
    default:
        al[0] = xi; al[1] = xi * e1 * (1. - e2); al[2] = xi * (1. - e1 * e2 * e3); al[3] = xi * e1 * (1. - e2 * e3);
        break;
    }
    return pow(xi, 3) * sq(e1) * e2;
}

void initializeQuadrule(Quad &q, const Mesh &m, const double *Pg) {
    const int nTr[3] = {2, 5, 6};
    for (int c = 0; c < 3; c++) {
        q.alphaC[c].assign((size_t)nTr[c] * q.nPg * 4, 0.0);
        q.tdetFrac[c].assign((size_t)nTr[c] * q.nPg, 0.0);
        q.alphaU[c].assign((size_t)nTr[c] * q.nPg * 4, 0.0);
        q.tdetWeak[c].assign((size_t)nTr[c] * q.nPg, 0.0);
        for (int t = 0; t < nTr[c]; t++) {
            for (int k = 0; k < q.nPg; k++) {
                double *al = &q.alphaC[c][((size_t)t * q.nPg + k) * 4];
                for (int j = 0; j < 4; j++) al[j] = Pg[4 * k + j];
                for (int j = 0; j < 4; j++) al[j] = al[j] * 0.5 + 0.5;        // scale()
                double *au = &q.alphaU[c][((size_t)t * q.nPg + k) * 4];
                for (int j = 0; j < 4; j++) au[j] = al[j];
                double tdw = pow(al[0], 3 - 2 - 2 * m.frac_s);
                double tdf = pow(al[0], 3 - 2 * m.frac_s);
                al[0] = 1.0;
                traffo(c, t, au);
                double det = traffo(c, t, al);
                tdw *= det * SCALEDET;
                tdf *= det * SCALEDET;
                al[0] = al[0] - al[1];                                         // mirror()
                al[2] = al[2] - al[3];
                au[0] = au[0] - au[1];
                au[2] = au[2] - au[3];
                q.tdetFrac[c][(size_t)t * q.nPg + k] = tdf;
                q.tdetWeak[c][(size_t)t * q.nPg + k] = tdw;
            }
        }
    }
}

// ---------------------------------------------------------------- dual graph (METIS_MeshToDual, ncommon=1)
void dual_graph(const Mesh &m, std::vector<long> &xadj, std::vector<long> &adj) {
    std::vector<long> vcnt(m.nV + 1, 0);
    for (long e = 0; e < m.nE; e++)
        for (int k = 0; k < m.dV; k++) vcnt[m.T[m.dV * e + k] + 1]++;
    for (long v = 0; v < m.nV; v++) vcnt[v + 1] += vcnt[v];
    std::vector<long> vel(vcnt[m.nV]);
    std::vector<long> fill(vcnt.begin(), vcnt.end() - 1);
    for (long e = 0; e < m.nE; e++)
        for (int k = 0; k < m.dV; k++) vel[fill[m.T[m.dV * e + k]]++] = e;
    xadj.assign(m.nE + 1, 0);
    adj.clear();
    std::vector<long> nb;
    for (long e = 0; e < m.nE; e++) {
        nb.clear();
        for (int k = 0; k < m.dV; k++) {
            long v = m.T[m.dV * e + k];
            for (long j = vcnt[v]; j < vcnt[v + 1]; j++)
                if (vel[j] != e) nb.push_back(vel[j]);
        }
        std::sort(nb.begin(), nb.end());
        nb.erase(std::unique(nb.begin(), nb.end()), nb.end());
        adj.insert(adj.end(), nb.begin(), nb.end());
        xadj[e + 1] = (long)adj.size();
    }
}

// ---------------------------------------------------------------- outdim > 1 (vector-valued kernels)
// The routines above with the reference's general indexing: blocks are (dV outdim) x (dV outdim),
// row index = vertex * outdim + component, kernel values row-major outdim x outdim. Only used
// when outdim > 1; the scalar routines are their outdim = 1 case written out.
int integrate_retriangulate_vec(const Elem &aT, const Elem &bT, const Quad &q, const Mesh &m,
                                double *tL, double *tN, double *tLP, double *tNP) {  // integration.cpp:345-540
    const int dV = 3, od = m.outdim, o2 = od * od, nB = dV * od;
    double x[2], y[2], ref[2], psi[3], kv[9], kvP[9];
    double innerLocal[9], innerNonloc[27], innerNonlocPrime[27];
    double reTri[9 * 3 * 2];
    int doesInteract = 0;
    for (int k = 0; k < q.nPx; k++) {
        toPhys(aT.E, &q.Px[2 * k], 2, x);
        const int Rdx = retri_method(m, x, bT.E, reTri);
        doesInteract += Rdx;
        for (int o = 0; o < o2; o++) innerLocal[o] = 0;
        for (int b = 0; b < dV * o2; b++) { innerNonloc[b] = 0; innerNonlocPrime[b] = 0; }
        for (int r = 0; r < Rdx; r++) {
            for (int i = 0; i < q.nPy; i++) {
                toPhys3(&reTri[6 * r], &q.Py[2 * i], y);
                const double rTdet = absDet2(&reTri[6 * r]);
                kernel_vec(m, x, aT.label, y, bT.label, kv);
                for (int o = 0; o < o2; o++) innerLocal[o] += kv[o] * q.dy[i] * rTdet;
                toRef(bT.E, y, ref);
                kernel_vec(m, y, bT.label, x, aT.label, kvP);
                basis(ref, 2, psi);
                for (int b = 0; b < dV * o2; b++) {
                    innerNonloc[b] += psi[b / o2] * kv[b % o2] * q.dy[i] * rTdet;
                    innerNonlocPrime[b] += psi[b / o2] * kvP[b % o2] * q.dy[i] * rTdet;
                }
                for (int a = 0; a < dV; a++)
                    for (int b = 0; b < dV; b++)
                        for (int o = 0; o < o2; o++)
                            tLP[a * o2 * dV + (o / od) * od * dV + b * od + o % od] +=
                                psi[a] * psi[b] * kvP[o] * q.dy[i] * q.dx[k] * rTdet * aT.absDet;
            }
        }
        for (int a = 0; a < nB; a++)
            for (int b = 0; b < nB; b++) {
                tL[nB * a + b] += aT.absDet * q.psix[dV * k + a / od] * q.psix[dV * k + b / od] * q.dx[k] *
                                  innerLocal[od * (a % od) + (b % od)];
                tN[nB * a + b] += aT.absDet * q.psix[dV * k + a / od] * q.dx[k] *
                                  innerNonloc[(a % od) * od + o2 * (b / od) + (b % od)];
                tNP[nB * a + b] += aT.absDet * q.psix[dV * k + a / od] * q.dx[k] *
                                   innerNonlocPrime[(a % od) * od + o2 * (b / od) + (b % od)];
            }
    }
    return (doesInteract || m.full_search);
}

int integrate_baryCenter_vec(const Elem &aT, const Elem &bT, const Quad &q, const Mesh &m,
                             double *tL, double *tN) {                       // integration.cpp:910-1018
    const int dim = m.dim, dV = m.dV, od = m.outdim, o2 = od * od, nB = dV * od;
    double x[3], y[3], kv[9], innerLocal[9], innerNonloc[36];
    int doesInteract = 0;
    for (int k = 0; k < q.nPx; k++) {
        toPhys(aT.E, &q.Px[dim * k], dim, x);
        for (int o = 0; o < o2; o++) innerLocal[o] = 0;
        for (int b = 0; b < dV * o2; b++) innerNonloc[b] = 0;
        const int Rdx = method_baryCenter(x, bT, m);
        doesInteract += Rdx;
        if (Rdx) {
            for (int i = 0; i < q.nPy; i++) {
                toPhys(bT.E, &q.Py[dim * i], dim, y);
                const double rTdet = absDetDim(bT.E, dim);
                kernel_vec(m, x, aT.label, y, bT.label, kv);
                for (int o = 0; o < o2; o++) innerLocal[o] += rTdet * kv[o] * q.dy[i];
                kernel_vec(m, y, bT.label, x, aT.label, kv);
                for (int b = 0; b < dV * o2; b++) innerNonloc[b] += q.psiy[dV * i + b / o2] * kv[b % o2] * q.dy[i] * rTdet;
            }
        }
        for (int a = 0; a < nB; a++)
            for (int b = 0; b < nB; b++) {
                tL[nB * a + b] += 2 * aT.absDet * q.psix[dV * k + a / od] * q.psix[dV * k + b / od] * q.dx[k] *
                                  innerLocal[od * (a % od) + (b % od)];
                tN[nB * a + b] += 2 * aT.absDet * q.psix[dV * k + a / od] * q.dx[k] *
                                  innerNonloc[(a % od) * od + o2 * (b / od) + (b % od)];
            }
    }
    return (doesInteract || m.full_search);
}

int integrate_weakSingular_vec(const Elem &aT, const Elem &bT, const Quad &q, const Mesh &m,
                               double *tL, double *tN, double *tLP, double *tNP) {  // integration.cpp:82-185
    Elem aS, bS;
    int argA[3], argB[3];
    const int nEqual = join(aT, bT, m, aS, bS, argA, argB);
    if (nEqual < 1 || nEqual > 3) return -1;  // reference aborts
    const int c = nEqual - 1;
    const int nT = (nEqual == 1) ? 2 : (nEqual == 2 ? 5 : 6);
    const int dV = 3, od = m.outdim;
    double xc[2], yc[2], psix[3], psiy[3], kv[9];
    for (int t = 0; t < nT; t++) {
        for (int k = 0; k < q.nPg; k++) {
            const double tw = q.tdetWeak[c][t * q.nPg + k];
            const double *ac = &q.alphaC[c][(t * q.nPg + k) * 4];
            const double *au = &q.alphaU[c][(t * q.nPg + k) * 4];
            toPhys(aS.E, &ac[0], 2, xc);
            toPhys(bS.E, &ac[2], 2, yc);
            kernel_vec(m, xc, aT.label, yc, bT.label, kv);
            basis(&au[0], 2, psix);
            basis(&au[2], 2, psiy);
            for (int a = 0; a < dV; a++)
                for (int aOut = 0; aOut < od; aOut++)
                    for (int b = 0; b < dV; b++)
                        for (int bOut = 0; bOut < od; bOut++) {
                            const double f = kv[od * aOut + bOut] * tw * q.dg[k] * aS.absDet * bS.absDet;
                            tL[od * dV * (argA[a] * od + aOut) + argA[b] * od + bOut] += f * psix[a] * psix[b];
                            tLP[od * dV * (argB[a] * od + aOut) + argB[b] * od + bOut] += f * psiy[a] * psiy[b];
                            tN[od * dV * (argA[a] * od + aOut) + argB[b] * od + bOut] += f * psix[a] * psiy[b];
                            tNP[od * dV * (argA[a] * od + aOut) + argB[b] * od + bOut] += f * psix[a] * psiy[b];
                        }
        }
    }
    return 1;
}

int integrate_fractional_vec(const Elem &aT, const Elem &bT, const Quad &q, const Mesh &m,
                             double *tL, double *tN, double *tLP, double *tNP) {  // integration.cpp:187-288
    Elem aS, bS;
    int argA[3], argB[3];
    const int nEqual = join(aT, bT, m, aS, bS, argA, argB);
    if (nEqual < 1 || nEqual > 3) return -1;  // reference aborts
    const int c = nEqual - 1;
    const int nT = (nEqual == 1) ? 2 : (nEqual == 2 ? 5 : 6);
    const int dV = 3, od = m.outdim, nLocal = 2 * dV - nEqual, shift = dV - nEqual;
    double x[2], y[2], psix[3], psiy[3], psixy[6], kv[9];
    for (int t = 0; t < nT; t++) {
        for (int k = 0; k < q.nPg; k++) {
            const double tf = q.tdetFrac[c][t * q.nPg + k];
            const double *al = &q.alphaC[c][(t * q.nPg + k) * 4];
            toPhys(aS.E, &al[0], 2, x);
            toPhys(bS.E, &al[2], 2, y);
            kernel_vec(m, x, aT.label, y, bT.label, kv);
            basis(&al[0], 2, psix);
            basis(&al[2], 2, psiy);
            for (int a = 0; a < nEqual; a++) psixy[a] = psix[a] - psiy[a];
            for (int a = nEqual; a < dV; a++) {
                psixy[a] = psix[a];
                psixy[a + shift] = -psiy[a];
            }
            for (int a = 0; a < nLocal; a++)
                for (int aOut = 0; aOut < od; aOut++)
                    for (int b = 0; b < nLocal; b++)
                        for (int bOut = 0; bOut < od; bOut++) {
                            const double f = kv[od * aOut + bOut] * tf * psixy[a] * psixy[b] * q.dg[k] * aS.absDet * bS.absDet;
                            if (a < dV) {
                                if (b < dV) tL[od * dV * (argA[a] * od + aOut) + argA[b] * od + bOut] += f;
                                else tN[od * dV * (argA[a] * od + aOut) + argB[b - shift] * od + bOut] -= f;
                            } else {
                                if (b < dV) tNP[od * dV * (argA[b] * od + aOut) + argB[a - shift] * od + bOut] -= f;
                                else tLP[od * dV * (argB[a - shift] * od + aOut) + argB[b - shift] * od + bOut] += f;
                            }
                        }
        }
    }
    return 1;
}

// ---------------------------------------------------------------- integrate dispatch (integration.cpp:67-79)
int integrate_method(int method, const Elem &aT, const Elem &bT, const Quad &q, const Mesh &m,
                     double *tL, double *tN, double *tLP, double *tNP) {
    if (m.outdim > 1) {
        switch (method) {
        case M_RETRIANGULATE: case M_RETRI_LINF: return integrate_retriangulate_vec(aT, bT, q, m, tL, tN, tLP, tNP);
        case M_BARYCENTER: return integrate_baryCenter_vec(aT, bT, q, m, tL, tN);
        case M_FRACTIONAL: return integrate_fractional_vec(aT, bT, q, m, tL, tN, tLP, tNP);
        case M_WEAKSING: return integrate_weakSingular_vec(aT, bT, q, m, tL, tN, tLP, tNP);
        }
        return -1;
    }
    switch (method) {
    case M_RETRIANGULATE: return integrate_retriangulate(aT, bT, q, m, tL, tN, tLP, tNP);
    case M_BARYCENTER: return integrate_baryCenter(aT, bT, q, m, tL, tN);
    case M_FRACTIONAL: return integrate_fractional(aT, bT, q, m, tL, tN, tLP, tNP);
    case M_RETRI_UNSYMM: return integrate_retriangulate_unsymm(aT, bT, q, m, tL, tN);
    case M_SUBSET: case M_AVERAGE: return integrate_subSuperSetBalls(aT, bT, q, m, method, tL, tN);
    case M_BARY_RT: return integrate_baryCenterRT(aT, bT, q, m, tL, tN);
    case M_NOTRUNC: return integrate_fullyContained(aT, bT, q, m, tL, tN, tLP, tNP);
    case M_WEAKSING: return integrate_weakSingular(aT, bT, q, m, tL, tN, tLP, tNP);
    case M_EXACT: return integrate_exact(aT, bT, q, m, tL, tN);
    case M_RETRI_LINF: return integrate_retriangulate(aT, bT, q, m, tL, tN, tLP, tNP);
    case M_UNSYMM_LINF: return integrate_retriangulate_unsymm(aT, bT, q, m, tL, tN);
    }
    return -1;
}
int integrate(const Elem &aT, const Elem &bT, const Quad &q, const Mesh &m, bool first,
              double *tL, double *tN, double *tLP, double *tNP) {
    return integrate_method(first ? m.close : m.remote, aT, bT, q, m, tL, tN, tLP, tNP);
}

// evaluateZeta (mathhelpers.cpp:19-38): the number of subdomains the two elements share, the
// size of the intersection of their sorted indicator rows.
double evaluateZeta(const long *ind, const long *ptr, long nColumns, long aTdx, long bTdx) {
    const long *a0 = &ind[ptr[aTdx]], *a1 = &ind[ptr[aTdx + 1]];
    const long *b0 = &ind[ptr[bTdx]], *b1 = &ind[ptr[bTdx + 1]];
    std::vector<long> inter((size_t)nColumns);
    auto ls = std::set_intersection(a0, a1, b0, b1, inter.begin());
    return (double)(ls - inter.begin());
}

struct Counters {
    long n_pairs = 0, n_cand = 0, n_close = 0, err = 0;
};

// One outer element: BFS over the dual graph, integrate each candidate, scatter the four local
// blocks, weighted by 1/zeta under domain decomposition, into the map. Cassemble.cpp:555-784
// (outdim = 1).
void system_element(long aTdx, const Mesh &m, const Quad &q, const std::vector<long> &xadj,
                    const std::vector<long> &adj, std::vector<int> &visited,
                    std::map<unsigned long, double> &Ad, Counters &cnt, std::vector<long> *pairs) {
    const int dV = m.dV;
    const unsigned long K = (unsigned long)m.K;
    long aDG[4], bDG[4];
    const long *aAdx, *bAdx;
    Elem aT, bT;
    double tL[144], tN[144], tLP[144], tNP[144];   // (dV outdim)^2, outdim <= 3
    const int od = m.outdim, nB = dV * od;
    if (m.is_dg) { for (int j = 0; j < dV; j++) aDG[j] = dV * aTdx + j; aAdx = aDG; }
    else aAdx = &m.T[dV * aTdx];
    initializeElement(aTdx, m, aT);
    std::queue<long> queue;
    queue.push(aTdx);
    std::fill(visited.begin(), visited.end(), 0);                        // Cassemble.cpp:597
    bool first = m.is_singular;                                           // :600
    while (!queue.empty()) {
        long s = queue.front();
        queue.pop();
        long start = xadj[s], end = xadj[s + 1];
        for (long nT = -1; start + nT != end; nT++) {                     // :613-622
            long bTdx = (nT == -1) ? aTdx : adj[start + nT];
            if (!visited[bTdx]) {
                if (m.labT[bTdx]) {
                    initializeElement(bTdx, m, bT);
                    if (m.is_dg) { for (int j = 0; j < dV; j++) bDG[j] = dV * bTdx + j; bAdx = bDG; }
                    else bAdx = &m.T[dV * bTdx];
                    for (int i = 0; i < nB * nB; i++) { tL[i] = 0; tN[i] = 0; tLP[i] = 0; tNP[i] = 0; }
                    cnt.n_cand++;
                    if (first) cnt.n_close++;
                    int does = integrate(aT, bT, q, m, first, tL, tN, tLP, tNP);
                    if (does < 0) { cnt.err++; does = 0; }
                    if (does) {
                        queue.push(bTdx);                                 // :713
                        cnt.n_pairs++;
                        if (pairs) { pairs->push_back(aTdx); pairs->push_back(bTdx); }
                        double weight = 1.;                               // :649-657
                        if (m.nZeta) weight = 1. / evaluateZeta(m.zeta_indices, m.zeta_indptr, m.nZeta, aTdx, bTdx);
                        if (od > 1) {                                     // :721-770, general indices
                            for (int a = 0; a < nB; a++)
                                for (int b = 0; b < nB; b++) {
                                    const unsigned long ra = (unsigned long)(od * aAdx[a / od] + a % od);
                                    const unsigned long rb = (unsigned long)(od * bAdx[b / od] + b % od);
                                    if (m.is_dg || m.labV[aAdx[a / od]] > 0) {
                                        Ad[ra * K + od * aAdx[b / od] + b % od] += tL[nB * a + b] * weight;
                                        Ad[ra * K + od * bAdx[b / od] + b % od] += -tN[nB * a + b] * weight;
                                    }
                                    if (m.is_dg || m.labV[bAdx[b / od]] > 0) {
                                        Ad[rb * K + od * bAdx[a / od] + a % od] += tLP[nB * a + b] * weight;
                                        Ad[rb * K + od * aAdx[a / od] + a % od] += -tNP[nB * a + b] * weight;
                                    }
                                }
                        } else
                        for (int a = 0; a < dV; a++) {                    // :721-770
                            for (int b = 0; b < dV; b++) {
                                if (m.is_dg || m.labV[aAdx[a]] > 0) {
                                    Ad[(unsigned long)aAdx[a] * K + aAdx[b]] += tL[dV * a + b] * weight;
                                    Ad[(unsigned long)aAdx[a] * K + bAdx[b]] += -tN[dV * a + b] * weight;
                                }
                                if (m.is_dg || m.labV[bAdx[b]] > 0) {
                                    Ad[(unsigned long)bAdx[b] * K + bAdx[a]] += tLP[dV * a + b] * weight;
                                    Ad[(unsigned long)bAdx[b] * K + aAdx[a]] += -tNP[dV * a + b] * weight;
                                }
                            }
                        }
                    }
                } else {
                    queue.push(bTdx);                                     // :773-775
                }
            }
            visited[bTdx] = 1;                                            // :778
        }
        first = false;                                                    // :782
    }
}

int kernel_id(const char *s) {
    std::string k(s ? s : "");
    if (k == "constant") return K_CONSTANT;
    if (k == "parabola") return K_PARABOLA;
    if (k == "fractional") return K_FRACTIONAL;
    if (k == "constant3D") return K_CONSTANT3D;
    if (k == "labeled") return K_LABELED;
    if (k == "notch") return K_NOTCH;
    if (k == "labeledNotch") return K_LABELEDNOTCH;
    if (k == "labeledValve") return K_LABELEDVALVE;
    if (k == "constantTruncated") return K_CONSTTRUNC;
    if (k == "linearPrototypeMicroelastic") return K_LINPROTO;
    if (k == "constantField") return K_FIELD_CONST;
    if (k == "linearPrototypeMicroelasticField") return K_FIELD_PROTO;
    if (k == "linearPrototypeMicroelasticField3D") return K_FIELD_PROTO3D;
    if (k == "constantLinf2D") return K_CONSTLINF;
    return K_NONE;
}
int load_id(const char *s) {
    std::string k(s ? s : "");
    if (k == "linear") return F_LINEAR;
    if (k == "linear3D") return F_LINEAR3D;
    if (k == "constant") return F_CONSTANT;
    if (k == "gaussian") return F_GAUSSIAN;
    if (k == "jump") return F_JUMP;
    if (k == "tensorsin") return F_TENSORSIN;
    if (k == "linearField") return F_FIELD_LINEAR;
    if (k == "linearField3D") return F_FIELD_LINEAR3D;
    if (k == "constantRightField") return F_FIELD_RIGHT;
    if (k == "constantDownField") return F_FIELD_DOWN;
    if (k == "constantBothField") return F_FIELD_BOTH;
    return F_NONE;
}
int method_id(const char *s) {
    std::string k(s ? s : "");
    if (k == "retriangulate") return M_RETRIANGULATE;
    if (k == "baryCenter") return M_BARYCENTER;
    if (k == "fractional") return M_FRACTIONAL;
    if (k == "retriangulate_unsymm") return M_RETRI_UNSYMM;
    if (k == "subSetBall") return M_SUBSET;
    if (k == "averageBall") return M_AVERAGE;
    if (k == "baryCenterRT") return M_BARY_RT;
    if (k == "noTruncation") return M_NOTRUNC;
    if (k == "weakSingular") return M_WEAKSING;
    if (k == "exactBall") return M_EXACT;
    if (k == "retriangulateLinfty") return M_RETRI_LINF;
    if (k == "retriangulate_unsymmLinfty") return M_UNSYMM_LINF;
    return M_NONE;
}

}  // namespace

// ====================================================================== C interface (ctypes)
extern "C" {

struct oracle_result {
    long K, nnz;
    long *indptr, *indices;
    double *values;
    double *fd;
    long n_pairs, n_candidates, n_close, n_errors;
    long *pairs;   // (n_pairs, 2) in BFS order per outer element, outer elements ascending
    double seconds;
};

void oracle_free(oracle_result *r) {
    if (!r) return;
    free(r->indptr); free(r->indices); free(r->values); free(r->fd); free(r->pairs);
    free(r);
}

// Method retriangulation of one ball center against one triangle (integration.cpp:1775-1894).
int oracle_retriangulate(const double *x, const double *TE, double sqdelta, double *out, int caps) {
    return method_retriangulate(x, TE, sqdelta, out, caps);
}
int oracle_toRef(const double *E, const double *x, double *p) { return toRef(E, x, p); }

// Twin of par_assemble (Cassemble.cpp:360-462 -> par_system :464-855 / par_forcing :857-928),
// returning CSR and the load vector in memory. compute: "system" or "forcing".
// subset (optional): only these outer elements are processed (CPU baseline sampling).
// nthreads <= 1: canonical single-threaded order (one map, as the reference's 1-thread run).
// Domain-decomposition indicator for the next oracle_par_assemble call (nZeta = 0: none).
static const long *g_zeta_indices = nullptr, *g_zeta_indptr = nullptr;
static long g_nZeta = 0;
void oracle_set_zeta(const long *indices, const long *indptr, long nZeta) {
    g_zeta_indices = indices;
    g_zeta_indptr = indptr;
    g_nZeta = nZeta;
}

oracle_result *oracle_par_assemble(
    const char *compute, int K, const long *ptrTriangles, const long *ptrLabelTriangles,
    const double *ptrVerts, const long *ptrLabelVerts, int nE, int nV,
    const double *Px, int nPx, const double *dx, const double *Py, int nPy, const double *dy,
    double sqdelta, int is_DG, const char *kernel, const char *f, const char *method_remote,
    const char *method_close, int is_PlacePointOnCap, int dim, int outdim,
    const double *Pg, int degree, const double *dg, double fractional_s,
    int is_fullConnectedComponentSearch, int nthreads, const long *subset, long n_subset,
    int want_pairs) {
    Mesh m;
    m.dim = dim; m.dV = dim + 1; m.outdim = outdim; m.is_dg = is_DG;
    m.nE = nE; m.nV = nV; m.K = K;
    m.T = ptrTriangles; m.labT = ptrLabelTriangles; m.labV = ptrLabelVerts; m.V = ptrVerts;
    m.zeta_indices = g_zeta_indices; m.zeta_indptr = g_zeta_indptr; m.nZeta = g_nZeta;
    m.sqdelta = sqdelta; m.delta = sqrt(sqdelta); m.frac_s = fractional_s;
    m.kernel = kernel_id(kernel); m.load = load_id(f);
    m.remote = method_id(method_remote);
    m.close = method_id(method_close && method_close[0] ? method_close : method_remote);
    std::string kn(kernel ? kernel : "");
    m.is_singular = (kn == "fractional" || kn == "linearPrototypeMicroelastic" ||
                     kn == "linearPrototypeMicroelasticField");               // Cassemble.cpp:89-94
    m.caps = is_PlacePointOnCap; m.full_search = is_fullConnectedComponentSearch;
    m.linf = (m.remote == M_RETRI_LINF || m.remote == M_UNSYMM_LINF || m.close == M_RETRI_LINF || m.close == M_UNSYMM_LINF);
    // vector-valued kernels: retriangulate, baryCenter and the fractional close rule
    if (outdim < 1 || outdim > dim) return nullptr;
    if (outdim > 1 && std::string(compute ? compute : "") == "system") {
        auto ok = [](int mth) { return mth == M_RETRIANGULATE || mth == M_BARYCENTER || mth == M_FRACTIONAL || mth == M_WEAKSING; };
        if (!ok(m.remote) || !ok(m.close)) return nullptr;
    }

    Quad q;
    q.Px = Px; q.dx = dx; q.Py = Py; q.dy = dy; q.nPx = nPx; q.nPy = nPy;
    q.nPg = degree > 0 ? (int)pow(degree, dim * 2) : 0;                     // MeshTypes.h:155
    q.dg = dg;
    q.psix.resize((size_t)m.dV * nPx);
    q.psiy.resize((size_t)m.dV * (nPy > 0 ? nPy : 1));
    for (int h = 0; h < nPx; h++) basis(&Px[dim * h], dim, &q.psix[m.dV * h]);   // Cassemble.cpp:509-516
    for (int h = 0; h < nPy; h++) basis(&Py[dim * h], dim, &q.psiy[m.dV * h]);
    if (q.nPg > 0 && Pg) initializeQuadrule(q, m, Pg);

    oracle_result *r = (oracle_result *)calloc(1, sizeof(oracle_result));
    r->K = K;
    double t0 = 0;
#ifdef _OPENMP
    t0 = omp_get_wtime();
#endif
    std::string comp(compute ? compute : "");
    if (comp == "forcing") {
        // par_forcing (Cassemble.cpp:857-928), compute_f (:149-164)
        std::vector<double> fd(K, 0.0);
        for (long aTdx = 0; aTdx < nE; aTdx++) {
            if (m.labT[aTdx] > 0) {
                Elem aT;
                initializeElement(aTdx, m, aT);
                long aDG[4];
                const long *aAdx;
                if (m.is_dg) { for (int j = 0; j < m.dV; j++) aDG[j] = m.dV * aTdx + j; aAdx = aDG; }
                else aAdx = &m.T[m.dV * aTdx];
                double termf[12] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
                double x[3];
                // domain decomposition: 1 / zeta of the element with itself (Cassemble.cpp:901-908)
                const double weight = m.nZeta ? 1. / evaluateZeta(m.zeta_indices, m.zeta_indptr, m.nZeta, aTdx, aTdx) : 1.;
                if (outdim > 1) {                                                  // compute_f, outdim > 1
                    for (int a = 0; a < m.dV * outdim; a++)
                        for (int i = 0; i < nPx; i++) {
                            // a scalar forcing sets fo[0] only: the reference reads the rest
                            // uninitialized, here they are NaN
                            double fo[3] = {NAN, NAN, NAN};
                            toPhys(aT.E, &Px[dim * i], dim, x);
                            load_vec(m, x, fo);
                            termf[a] += q.psix[m.dV * i + a / outdim] * fo[a % outdim] * aT.absDet * dx[i];
                        }
                    for (int a = 0; a < m.dV * outdim; a++)
                        if (m.is_dg || m.labV[aAdx[a / outdim]] > 0) fd[outdim * aAdx[a / outdim] + a % outdim] += termf[a] * weight;
                    continue;
                }
                for (int a = 0; a < m.dV; a++) {
                    for (int i = 0; i < nPx; i++) {
                        toPhys(aT.E, &Px[dim * i], dim, x);
                        double fv = load_value(m, x);
                        termf[a] += q.psix[m.dV * i + a] * fv * aT.absDet * dx[i];
                    }
                }
                for (int a = 0; a < m.dV; a++)
                    if (m.is_dg || m.labV[aAdx[a]] > 0) fd[aAdx[a]] += termf[a] * weight;
            }
        }
        r->fd = (double *)malloc(sizeof(double) * K);
        memcpy(r->fd, fd.data(), sizeof(double) * K);
    } else {
        std::vector<long> xadj, adj;
        dual_graph(m, xadj, adj);
        std::vector<long> outer;
        if (subset) outer.assign(subset, subset + n_subset);
        else for (long e = 0; e < nE; e++) outer.push_back(e);
        int nt = nthreads > 1 ? nthreads : 1;
        std::vector<std::map<unsigned long, double>> maps(nt);
        std::vector<Counters> cnts(nt);
        std::vector<std::vector<long>> pairs(nt);
#ifdef _OPENMP
#pragma omp parallel num_threads(nt)
#endif
        {
            int tid = 0;
#ifdef _OPENMP
            tid = omp_get_thread_num();
#endif
            std::vector<int> visited(nE, 0);
            long n = (long)outer.size();
            long lo = n * tid / nt, hi = n * (tid + 1) / nt;  // contiguous element blocks
            for (long i = lo; i < hi; i++) {
                long aTdx = outer[i];
                if (m.labT[aTdx])                                          // Cassemble.cpp:559
                    system_element(aTdx, m, q, xadj, adj, visited, maps[tid], cnts[tid],
                                   want_pairs ? &pairs[tid] : nullptr);
            }
        }
        // merge thread maps, sum duplicates in thread order, drop exact zeros (arma::sp_mat)
        std::map<unsigned long, double> &all = maps[0];
        for (int t = 1; t < nt; t++)
            for (auto &it : maps[t]) all[it.first] += it.second;
        long nnz = 0;
        for (auto &it : all) if (it.second != 0.0) nnz++;
        r->nnz = nnz;
        r->indptr = (long *)calloc(K + 1, sizeof(long));
        r->indices = (long *)malloc(sizeof(long) * (nnz ? nnz : 1));
        r->values = (double *)malloc(sizeof(double) * (nnz ? nnz : 1));
        long k = 0;
        for (auto &it : all) {
            if (it.second == 0.0) continue;
            long row = (long)(it.first / (unsigned long)K), col = (long)(it.first % (unsigned long)K);
            r->indices[k] = col;
            r->values[k] = it.second;
            r->indptr[row + 1]++;
            k++;
        }
        for (long i = 0; i < K; i++) r->indptr[i + 1] += r->indptr[i];
        for (int t = 0; t < nt; t++) {
            r->n_pairs += cnts[t].n_pairs;
            r->n_candidates += cnts[t].n_cand;
            r->n_close += cnts[t].n_close;
            r->n_errors += cnts[t].err;
        }
        if (want_pairs) {
            r->pairs = (long *)malloc(sizeof(long) * 2 * (r->n_pairs ? r->n_pairs : 1));
            long o = 0;
            for (int t = 0; t < nt; t++) {
                memcpy(r->pairs + o, pairs[t].data(), sizeof(long) * pairs[t].size());
                o += (long)pairs[t].size();
            }
        }
    }
#ifdef _OPENMP
    r->seconds = omp_get_wtime() - t0;
#endif
    return r;
}

// Local blocks of explicit (aT, bT) pairs, for kernel-level parity tests.
// out: (n, 4, dV, dV) = termLocal, termNonloc, termLocalPrime, termNonlocPrime; ret[i] = doesInteract.
int oracle_pair_blocks(
    const long *ptrTriangles, const long *ptrLabelTriangles, const double *ptrVerts, int nE, int nV,
    const double *Px, int nPx, const double *dx, const double *Py, int nPy, const double *dy,
    double sqdelta, const char *kernel, const char *method, int is_PlacePointOnCap, int dim,
    const double *Pg, int degree, const double *dg, double fractional_s,
    const long *pairs, long n, double *out, int *ret) {
    Mesh m;
    memset(&m, 0, sizeof(m));
    m.dim = dim; m.dV = dim + 1; m.outdim = 1;
    m.nE = nE; m.nV = nV; m.T = ptrTriangles; m.labT = ptrLabelTriangles; m.V = ptrVerts;
    m.sqdelta = sqdelta; m.delta = sqrt(sqdelta); m.frac_s = fractional_s;
    m.kernel = kernel_id(kernel); m.caps = is_PlacePointOnCap;
    int meth = method_id(method);
    m.linf = (meth == M_RETRI_LINF || meth == M_UNSYMM_LINF);
    Quad q;
    q.Px = Px; q.dx = dx; q.Py = Py; q.dy = dy; q.nPx = nPx; q.nPy = nPy;
    q.nPg = degree > 0 ? (int)pow(degree, dim * 2) : 0;
    q.dg = dg;
    q.psix.resize((size_t)m.dV * nPx);
    q.psiy.resize((size_t)m.dV * (nPy > 0 ? nPy : 1));
    for (int h = 0; h < nPx; h++) basis(&Px[dim * h], dim, &q.psix[m.dV * h]);
    for (int h = 0; h < nPy; h++) basis(&Py[dim * h], dim, &q.psiy[m.dV * h]);
    if (q.nPg > 0 && Pg) initializeQuadrule(q, m, Pg);
    const int bs = m.dV * m.dV;
    for (long i = 0; i < n; i++) {
        Elem aT, bT;
        initializeElement(pairs[2 * i], m, aT);
        initializeElement(pairs[2 * i + 1], m, bT);
        double *o = &out[i * 4 * bs];
        for (int j = 0; j < 4 * bs; j++) o[j] = 0;
        ret[i] = integrate_method(meth, aT, bT, q, m, o, o + bs, o + 2 * bs, o + 3 * bs);
    }
    return 0;
}

// par_evaluateMass (Cassemble.cpp:166-246): vd += psi_a psi_b |aT| dx_j ud over the first J
// elements with label > 0; CG rows and columns of vertices with label > 0, DG indices
// dV * aTdx + j; the (a, aOut, b, bOut, j) loop order of the reference, sequentially.
int oracle_evaluate_mass(double *vd, const double *ud, const long *Elements, const long *ElementLabels,
                         const double *Verts, const long *VertexLabels, int J, int nP, const double *P,
                         const double *dx, int dim, int outdim, int is_dg) {
    const int dVerts = dim + 1;
    std::vector<double> psi((size_t)dVerts * nP);
    double tmp[4];
    for (int k = 0; k < nP; k++) {
        basis(&P[dim * k], dim, tmp);
        for (int kk = 0; kk < dVerts; kk++) psi[(size_t)nP * kk + k] = tmp[kk];
    }
    long aDG[4];
    double aTE[12];
    for (int aTdx = 0; aTdx < J; aTdx++) {
        if (ElementLabels[aTdx] <= 0) continue;
        const long *aAdx;
        if (is_dg) {
            for (int j = 0; j < dVerts; j++) aDG[j] = (long)dVerts * aTdx + j;
            aAdx = aDG;
        } else {
            aAdx = &Elements[(long)dVerts * aTdx];
        }
        for (int jj = 0; jj < dVerts; jj++)
            for (int j = 0; j < dim; j++) aTE[dim * jj + j] = Verts[dim * Elements[(long)dVerts * aTdx + jj] + j];
        const double aTdet = absDetDim(aTE, dim);
        for (int a = 0; a < dVerts; a++) {
            if (!(is_dg || VertexLabels[aAdx[a]] > 0)) continue;
            for (int aOut = 0; aOut < outdim; aOut++)
                for (int b = 0; b < dVerts; b++) {
                    if (!(is_dg || VertexLabels[aAdx[b]] > 0)) continue;
                    for (int bOut = 0; bOut < outdim; bOut++)
                        for (int j = 0; j < nP; j++)
                            vd[outdim * aAdx[a] + aOut] +=
                                psi[(size_t)nP * a + j] * psi[(size_t)nP * b + j] * aTdet * dx[j] * ud[outdim * aAdx[b] + bOut];
                }
        }
    }
    return 0;
}

}  // extern "C"
