// Host orchestration of the assembly pipeline and the C ABI (included by assemble.cu).
#include <map>
#include <mutex>

namespace nlg {

static thread_local std::string g_err;
static thread_local nlfem_stats g_stats;

static int fail(int code, const std::string &msg) {
    g_err = msg;
    return code;
}

#define CK(call)                                                                       \
    do {                                                                               \
        cudaError_t e_ = (call);                                                       \
        if (e_ != cudaSuccess)                                                         \
            return fail(NLFEM_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

static inline unsigned grid_for(long long n, int threads) {
    long long g = (n + threads - 1) / threads;
    return (unsigned)(g < 1 ? 1 : g);
}

// Grow-only device buffer.
struct DevBuf {
    void *p = nullptr;
    size_t cap = 0;
    template <typename T>
    T *get() const { return (T *)p; }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        cap = 0;
    }
};

static int ensure(DevBuf &b, size_t bytes, bool no_grow) {
    if (bytes == 0) bytes = 16;
    if (bytes <= b.cap) return NLFEM_OK;
    // a captured sequence cannot allocate; the run before the capture sizes every buffer
    if (no_grow) return fail(NLFEM_ERR_CUDA, "internal: a buffer would grow during graph capture");
    size_t want = std::max(bytes, (size_t)(b.cap + b.cap / 4));   // a regrown buffer gets 25% headroom
    b.release();
    cudaError_t e = cudaMalloc(&b.p, want);
    if (e != cudaSuccess) {
        cudaGetLastError();
        e = cudaMalloc(&b.p, bytes);
        want = bytes;
    }
    if (e != cudaSuccess) {
        cudaGetLastError();
        b.p = nullptr;
        return fail(NLFEM_ERR_NOMEM, "cudaMalloc of " + std::to_string(bytes) + " bytes failed");
    }
    b.cap = want;
    return NLFEM_OK;
}
#define ENS(buf, bytes) do { int r_ = ensure(buf, bytes, S.replay); if (r_) return r_; } while (0)

// ---------------------------------------------------------------- configuration parsing
static int kernel_id(const char *s) {
    std::string k(s ? s : "");
    if (k == "constant") return KER_CONSTANT;
    if (k == "parabola") return KER_PARABOLA;
    if (k == "fractional") return KER_FRACTIONAL;
    if (k == "linearPrototypeMicroelastic") return KER_FRACTIONAL;   // c |z|^-1: exponent 1, see make_params
    if (k == "constant3D") return KER_CONSTANT3D;
    if (k == "labeled") return KER_LABELED;
    if (k == "notch") return KER_NOTCH;
    if (k == "labeledNotch") return KER_LABELEDNOTCH;
    if (k == "labeledValve") return KER_LABELEDVALVE;
    if (k == "constantTruncated") return KER_CONSTTRUNC;
    if (k == "constantField") return KER_CONSTFIELD;
    if (k == "linearPrototypeMicroelasticField") return KER_MICROFIELD;
    if (k == "linearPrototypeMicroelasticField3D") return KER_MICROFIELD3D;
    return -1;
}
static int method_id(const char *s) {
    std::string k(s ? s : "");
    if (k == "retriangulate") return MTH_RETRIANGULATE;
    if (k == "baryCenter") return MTH_BARYCENTER;
    if (k == "fractional") return MTH_FRACTIONAL;
    if (k == "weakSingular") return MTH_WEAKSING;
    if (k == "retriangulate_unsymm") return MTH_RETRI_UNSYMM;
    if (k == "subSetBall") return MTH_SUBSET;
    if (k == "averageBall") return MTH_AVERAGE;
    if (k == "baryCenterRT") return MTH_BARY_RT;
    if (k == "noTruncation") return MTH_NOTRUNC;
    if (k == "exactBall") return MTH_EXACT;
    return -1;
}
static int load_id(const char *s) {
    std::string k(s ? s : "");
    if (k == "linear") return LOAD_LINEAR;
    if (k == "linear3D") return LOAD_LINEAR3D;
    if (k == "constant") return LOAD_CONSTANT;
    if (k == "gaussian") return LOAD_GAUSSIAN;
    if (k == "jump") return LOAD_JUMP;
    if (k == "tensorsin") return LOAD_TENSORSIN;
    if (k == "linearField") return LOAD_LINEARFIELD;
    if (k == "linearField3D") return LOAD_LINEARFIELD3D;
    if (k == "constantRightField") return LOAD_RIGHTFIELD;
    if (k == "constantDownField") return LOAD_DOWNFIELD;
    if (k == "constantBothField") return LOAD_BOTHFIELD;
    return -1;
}
// Number of components of a kernel's or a forcing's values (model.cpp:140-191, 204-238).
static int kernel_outdim(int k) { return k == KER_MICROFIELD3D ? 3 : (k >= KER_CONSTFIELD ? 2 : 1); }
static int load_outdim(int l) {
    if (l == LOAD_LINEARFIELD3D) return 3;
    return l >= LOAD_LINEARFIELD ? 2 : 1;
}

// Quadrature rule and the basis function check (Cassemble.cpp:509-517, checks.cpp:36-47).
static int make_rule(const nlfem_problem &p, bool inner, Rule &r) {
    memset(&r, 0, sizeof(r));
    const int dim = p.dim, dV = dim + 1;
    r.dim = dim;
    r.nPx = p.nPx;
    r.nPy = inner ? p.nPy : 0;
    if (p.nPx <= 0 || p.nPx > MAXQ || !p.Px || !p.dx)
        return fail(NLFEM_ERR_INVALID, "outer quadrature rule missing or longer than 32 points");
    if (inner && (p.nPy <= 0 || p.nPy > MAXQ || !p.Py || !p.dy))
        return fail(NLFEM_ERR_INVALID, "inner quadrature rule missing or longer than 32 points");
    for (int k = 0; k < r.nPx; k++) {
        double s = 1.0;
        for (int j = 0; j < dim; j++) {
            r.Px[dim * k + j] = p.Px[dim * k + j];
            s -= p.Px[dim * k + j];
            r.psix[dV * k + j + 1] = p.Px[dim * k + j];
            r.Pxf[dim * k + j] = (float)p.Px[dim * k + j];
        }
        r.psix[dV * k] = s;
        r.dx[k] = p.dx[k];
    }
    for (int k = 0; k < r.nPy; k++) {
        double s = 1.0;
        for (int j = 0; j < dim; j++) {
            r.Py[dim * k + j] = p.Py[dim * k + j];
            s -= p.Py[dim * k + j];
            r.psiy[dV * k + j + 1] = p.Py[dim * k + j];
        }
        r.psiy[dV * k] = s;
        r.dy[k] = p.dy[k];
        for (int j = 0; j < dim && j < 2; j++) r.Pyf[2 * k + j] = (float)p.Py[dim * k + j];
        r.dyf[k] = (float)p.dy[k];
        for (int a = 0; a < dV; a++) r.psiyf[dV * k + a] = (float)r.psiy[dV * k + a];
    }
    // chk_BasisFunction: sum_k w_k psi_0(P_k) == 1/(d+1)!
    const double want = dim == 2 ? 1.0 / 6.0 : 1.0 / 24.0;
    double sx = 0;
    for (int k = 0; k < r.nPx; k++) sx += r.dx[k] * r.psix[dV * k];
    if (fabs(sx - want) >= 1e-8) return fail(NLFEM_ERR_INVALID, "Wrong integral of basis function w.r.t. weights dx.");
    if (inner) {
        double sy = 0;
        for (int k = 0; k < r.nPy; k++) sy += r.dy[k] * r.psiy[dV * k];
        if (fabs(sy - want) >= 1e-8) return fail(NLFEM_ERR_INVALID, "Wrong integral of basis function w.r.t. weights dy.");
    }
    return NLFEM_OK;
}

// Per-problem parameters, checks (checks.cpp:87-113) and the fixed-point scale.
// Unit of the 64-bit fixed-point CSR sums of the one-sided pass: entries up to 2^(scale_exp +
// FX_GUARD) fit; widen moves the unit up when a pass reported an out-of-range contribution.
static int set_fx_unit(ProbParams &P, int widen) {
    P.fx_ue = P.scale_exp + FX_GUARD - 62 + widen;
    if (P.fx_ue <= -120 || P.fx_ue >= 120)
        return fail(NLFEM_ERR_UNSUPPORTED, "matrix entries outside the range of the fixed-point accumulation");
    P.fx_unit = std::ldexp(1.0, P.fx_ue);
    P.fx_mul = std::ldexp(1.0f, -P.fx_ue);
    return NLFEM_OK;
}

// Number of subdomains elements a and b share: the sorted-merge intersection of their indicator
// rows (evaluateZeta, mathhelpers.cpp:19-37).
static long zeta_common(const long *idx, const long *ptr, long a, long b) {
    long i = ptr[a], ie = ptr[a + 1], j = ptr[b], je = ptr[b + 1], n = 0;
    while (i < ie && j < je) {
        if (idx[i] < idx[j]) i++;
        else if (idx[j] < idx[i]) j++;
        else { n++; i++; j++; }
    }
    return n;
}

static int make_params(const nlfem_problem &p, bool system, ProbParams &P) {
    memset(&P, 0, sizeof(P));
    if (p.dim != 2 && p.dim != 3) return fail(NLFEM_ERR_INVALID, "Dimension is not equal to 2 or 3.");
    if (p.outdim < 1 || p.outdim > 3) return fail(NLFEM_ERR_INVALID, "outdim must be 1, 2 or 3");
    if (p.is_dg && (long long)(p.dim + 1) * p.nE >= (1LL << 31)) return fail(NLFEM_ERR_UNSUPPORTED, "mesh too large for DG");
    if (p.nE <= 0 || p.nV <= 0 || !p.elements || !p.elementLabels || !p.vertices || !p.vertexLabels)
        return fail(NLFEM_ERR_INVALID, "empty or missing mesh arrays");
    if (p.nE >= (1LL << 31) || p.nV >= (1LL << 31)) return fail(NLFEM_ERR_UNSUPPORTED, "mesh too large");
    P.sqdelta = p.sqdelta;
    P.delta = sqrt(p.sqdelta);
    P.sqdelta_f = (float)p.sqdelta;
    if (system) {
        P.kernel = kernel_id(p.kernel);
        if (P.kernel < 0) return fail(NLFEM_ERR_UNSUPPORTED, std::string("unknown kernel: ") + (p.kernel ? p.kernel : "(null)"));
        P.remote = method_id(p.method_remote);
        P.close = (p.method_close && p.method_close[0]) ? method_id(p.method_close) : P.remote;
        if (P.remote < 0 || P.close < 0) return fail(NLFEM_ERR_UNSUPPORTED, "unknown integration method");
        if (p.dim == 3 && P.remote != MTH_BARYCENTER)
            return fail(NLFEM_ERR_INVALID, "Only Bary-Center is currently implemented as integration method for 3D and 1D.");
        if (P.remote == MTH_FRACTIONAL || P.remote == MTH_WEAKSING)
            return fail(NLFEM_ERR_INVALID, "The fractional and fractional_weakSingular integration routines are meant for close elements only.");
        std::string kn(p.kernel);
        const bool proto = kn == "linearPrototypeMicroelastic";
        // chk_Conf (checks.cpp:105-113)
        if (P.close == MTH_FRACTIONAL && p.is_dg)
            return fail(NLFEM_ERR_INVALID, "The fractional integration routine cannot be used for DG ansatz spaces. Try "
                                           "using the weakSingular integration routine if your singularity is of degree "
                                           "2+2s for s<=0.5.");
        if ((proto || kn == "linearPrototypeMicroelasticField") && p.fractional_s != -0.5)
            return fail(NLFEM_ERR_INVALID, "The fractional_s corresponding to the linearPrototypeMicroelastic kernels is "
                                           "s=-0.5, as 2+2s = 1. Please set fractional_s.");
        P.singular = (kn == "fractional") || proto || P.kernel == KER_MICROFIELD;   // Cassemble.cpp:89-94
        if (kernel_outdim(P.kernel) != p.outdim)
            return fail(NLFEM_ERR_INVALID, std::string("kernel ") + kn + " has " + std::to_string(kernel_outdim(P.kernel)) +
                                               " output components, outdim is " + std::to_string(p.outdim));
        if (p.outdim > 1) {   // vector-valued kernels: the FP64 vector path
            if (p.dim != (P.kernel == KER_MICROFIELD3D ? 3 : 2))
                return fail(NLFEM_ERR_INVALID, std::string("kernel ") + kn + " needs a " +
                                                   (P.kernel == KER_MICROFIELD3D ? "3D" : "2D") + " mesh");
            if (p.precision != NLFEM_PREC_FP64)
                return fail(NLFEM_ERR_UNSUPPORTED, "vector-valued kernels run on the fp64 path only (precision \"fp64\")");
            if (p.is_dg) return fail(NLFEM_ERR_UNSUPPORTED, "the DG ansatz with vector-valued kernels is not implemented");
            if (p.nZeta > 0)
                return fail(NLFEM_ERR_UNSUPPORTED, "domain-decomposition weights with vector-valued kernels are not implemented");
            if ((P.remote != MTH_RETRIANGULATE && P.remote != MTH_BARYCENTER) ||
                (P.close != MTH_RETRIANGULATE && P.close != MTH_BARYCENTER && P.close != MTH_FRACTIONAL && P.close != MTH_WEAKSING))
                return fail(NLFEM_ERR_UNSUPPORTED, "vector-valued kernels take retriangulate or baryCenter (remote) and "
                                                   "those or fractional / weakSingular (close)");
        }
        if (proto && p.dim != 2) return fail(NLFEM_ERR_UNSUPPORTED, "kernel linearPrototypeMicroelastic is implemented for 2D meshes only");
        if (duffy_close(P) && (p.tensorGaussDegree <= 0 || !p.Pg || !p.dg))
            return fail(NLFEM_ERR_INVALID, "You chose an integration routing for singular kernels, but no quadrature rule for it.");
        if ((P.close == MTH_FRACTIONAL || P.close == MTH_WEAKSING) && p.dim != 2)
            return fail(NLFEM_ERR_UNSUPPORTED, "fractional and weakSingular close pairs are 2D only");
        if (P.singular && P.close == MTH_WEAKSING && p.precision == NLFEM_PREC_FP64_ONESIDED)
            return fail(NLFEM_ERR_UNSUPPORTED, "precision \"fp64-onesided\" takes the fractional close rule only");
        if (p.dim == 2 && (P.kernel == KER_CONSTANT3D)) return fail(NLFEM_ERR_INVALID, "constant3D kernel needs a 3D mesh");
        if (p.is_dg && p.precision != NLFEM_PREC_FP64)
            return fail(NLFEM_ERR_UNSUPPORTED, "the DG ansatz runs on the fp64 path only (precision \"fp64\")");
        if ((P.remote >= MTH_RETRI_UNSYMM || (P.close >= MTH_RETRI_UNSYMM && P.close != MTH_WEAKSING)) &&
            p.precision != NLFEM_PREC_FP64)
            return fail(NLFEM_ERR_UNSUPPORTED, std::string("integration method ") +
                        (P.remote >= MTH_RETRI_UNSYMM ? p.method_remote : p.method_close) + " runs on the fp64 path only (precision \"fp64\")");
        if (P.kernel >= KER_LABELED && P.kernel <= KER_CONSTTRUNC) {   // label- or position-dependent kernels of 2D meshes
            if (p.dim != 2) return fail(NLFEM_ERR_UNSUPPORTED, std::string("kernel ") + p.kernel + " is implemented for 2D meshes only");
            if (p.precision != NLFEM_PREC_FP64)
                return fail(NLFEM_ERR_UNSUPPORTED, std::string("kernel ") + p.kernel + " runs on the fp64 path only (precision \"fp64\")");
        }
        P.caps = p.is_PlacePointOnCap ? 1 : 0;
        P.full_search = p.is_fullConnectedComponentSearch ? 1 : 0;
        const double s = p.fractional_s;
        switch (P.kernel) {
        case KER_CONSTANT: P.kc = 4 / (M_PI * (p.sqdelta * p.sqdelta)); break;             // model.cpp:25-28
        case KER_PARABOLA: P.kc = 12. / (M_PI * pow(p.sqdelta, 3)); break;                 // model.cpp:52-60
        case KER_FRACTIONAL:
            if (proto) {   // model.cpp:116-124: 3 / (pi delta^3) / |z|; the Duffy tables keep s
                P.expo = 1.0;
                P.kc = 3.0 / (M_PI * pow(P.delta, 3));
            } else {       // model.cpp:126-138
                P.expo = p.dim + 2. * s;
                P.kc = (2. - 2. * s) / (M_PI * pow(P.delta, 2. - 2. * s));
            }
            break;
        case KER_CONSTANT3D: P.kc = 15 / (M_PI * 4 * pow(P.delta, 5)); break;              // model.cpp:62-65
        case KER_LABELED:                                                                  // model.cpp:67-89
            P.kc = 0.01 * 3. / (4 * pow(p.sqdelta, 2));
            P.kc2 = 100 * 3. / (4 * pow(p.sqdelta, 2));
            break;
        case KER_NOTCH: case KER_LABELEDNOTCH: case KER_LABELEDVALVE:                      // model.cpp:91-114
            P.kc = 4 / (M_PI * pow(p.sqdelta, 2));
            break;
        case KER_CONSTTRUNC: P.kc = 4 / (M_PI * pow(p.sqdelta, 2)); break;                 // model.cpp:30-42
        case KER_CONSTFIELD: P.kc = 4. / (M_PI * pow(p.sqdelta, 2)); break;                // model.cpp:182-191
        case KER_MICROFIELD: case KER_MICROFIELD3D:                                        // model.cpp:140-180
            P.kc = 3.0 / pow(P.delta, 3);
            P.expo = 1.0;   // |k| ~ c / |z|: for the fixed-point scale
            break;
        }
        P.kc_f = (float)P.kc;
        P.expo_f = (float)P.expo;
    } else {
        P.load = load_id(p.forcing);
        if (P.load < 0) return fail(NLFEM_ERR_UNSUPPORTED, std::string("unknown forcing: ") + (p.forcing ? p.forcing : "(null)"));
        if (load_outdim(P.load) != p.outdim)
            return fail(NLFEM_ERR_INVALID, std::string("forcing ") + p.forcing + " has " + std::to_string(load_outdim(P.load)) +
                                               " components, outdim is " + std::to_string(p.outdim));
        if (p.outdim > 1 && p.is_dg) return fail(NLFEM_ERR_UNSUPPORTED, "the DG ansatz with vector forcings is not implemented");
    }
    P.bridges = 0;
    if (p.elementLabels)
        for (long e = 0; e < p.nE && !P.bridges; e++) P.bridges = p.elementLabels[e] == 0;
    P.zeta = 0;
    if (p.nZeta > 0) {   // the device reads the indicator rows by these pointers
        if (!p.zeta_indices || !p.zeta_indptr) return fail(NLFEM_ERR_INVALID, "nZeta > 0 without the zeta indicator");
        if (p.zeta_indptr[0] != 0) return fail(NLFEM_ERR_INVALID, "zeta indicator: row pointers must start at 0");
        for (long e = 0; e < p.nE; e++)
            if (p.zeta_indptr[e + 1] < p.zeta_indptr[e]) return fail(NLFEM_ERR_INVALID, "zeta indicator: decreasing row pointers");
        if (system) {   // chk_Mesh (checks.cpp:74-84): the first 20 elements share a subdomain pairwise
            const long m = std::min<long>(p.nE, 20);
            for (long k = 0; k < m; k++)
                for (long j = 0; j < m; j++)
                    if (zeta_common(p.zeta_indices, p.zeta_indptr, k, j) == 0)
                        return fail(NLFEM_ERR_INVALID, "Some rows Zeta(k).dot(Zeta(j)) evaluate to zero.");
        }
        P.zeta = 1;
    }
    // fixed-point scale: typical magnitude of an entry
    double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
    for (long v = 0; v < p.nV; v++)
        for (int j = 0; j < p.dim; j++) {
            double x = p.vertices[v * p.dim + j];
            lo[j] = std::min(lo[j], x);
            hi[j] = std::max(hi[j], x);
        }
    double vol = 1;
    for (int j = 0; j < p.dim; j++) vol *= std::max(hi[j] - lo[j], 1e-300);
    const double el = vol / (double)p.nE;
    P.el = el;
    // The one-sided passes decide their geometry with margins (certified.cuh; 2^-40 for the FP64
    // instance). The rounding of coordinates local to an outer element grows with the element
    // size relative to the ball: the FP32 vertex tests stay inside their margin while every element
    // diameter is at most MIX_MAX_H_OVER_DELTA times delta (the FP64 ones up to 512 delta).
    if (system && (p.precision == NLFEM_PREC_MIXED || p.precision == NLFEM_PREC_FP64_ONESIDED)) {
        const int dV = p.dim + 1;
        double hmax2 = 0;
        for (long e = 0; e < p.nE; e++)
            for (int a = 0; a < dV; a++)
                for (int b = a + 1; b < dV; b++) {
                    const long va = p.elements[e * dV + a], vb = p.elements[e * dV + b];
                    if (va < 0 || vb < 0 || va >= p.nV || vb >= p.nV) continue;   // rejected by the mesh checks
                    double d2 = 0;
                    for (int j = 0; j < p.dim; j++) {
                        const double d = p.vertices[va * p.dim + j] - p.vertices[vb * p.dim + j];
                        d2 += d * d;
                    }
                    hmax2 = std::max(hmax2, d2);
                }
        const double lim = p.precision == NLFEM_PREC_MIXED ? MIX_MAX_H_OVER_DELTA : 512.0;
        if (hmax2 > lim * lim * p.sqdelta)
            return fail(NLFEM_ERR_UNSUPPORTED, std::string("precision \"") + (p.precision == NLFEM_PREC_MIXED ? "mixed" : "fp64-onesided") +
                        "\" needs elements no larger than " + std::to_string((int)lim) +
                        " times the horizon (the margins of its geometry tests); precision \"fp64\" has no such bound");
    }
    double mag;
    if (system) {
        const double h = pow(el, 1.0 / p.dim);
        const double ball = p.dim == 2 ? M_PI * p.sqdelta : 4.0 / 3.0 * M_PI * p.sqdelta * P.delta;
        double kmax = P.kc;
        if (P.kernel == KER_PARABOLA) kmax = P.kc * p.sqdelta;
        if (P.kernel == KER_LABELED) kmax = std::max(P.kc, P.kc2);
        if (P.kernel == KER_FRACTIONAL || P.kernel == KER_MICROFIELD || P.kernel == KER_MICROFIELD3D)
            kmax = P.kc / pow(std::min(h, P.delta), P.expo);
        mag = fabs(kmax) * el * std::max(ball, el);
    } else {
        double fm = 1.0;
        for (int j = 0; j < p.dim; j++) fm = std::max(fm, std::max(fabs(lo[j]), fabs(hi[j])));
        mag = 2.0 * (fm + 2.0) * el;
    }
    if (!(mag > 0) || !std::isfinite(mag)) mag = 1.0;
    P.scale_exp = exact_ceil_log2(mag);
    return set_fx_unit(P, 0);
}

// Duffy tables (MeshTypes.cpp:32-209, 252-327): scaled points, xi factored out of the transform
// (alphaCanceled[0] = 1), determinant xi^(3-2s) * traffoDet * SCALEDET, mirrored.
static double duffy_traffo(int c, int t, double *al) {
    const double xi = al[0], e1 = al[1], e2 = al[2], e3 = al[3];
    if (c == 0) {
        if (t == 0) { al[0] = xi; al[1] = e1 * xi; al[2] = e2 * xi; al[3] = e2 * e3 * xi; }
        else { al[0] = xi * e2; al[1] = xi * e2 * e3; al[2] = xi; al[3] = xi * e1; }
        return pow(xi, 3) * e2;
    }
    if (c == 1) {
        switch (t) {
        case 0: al[0] = xi; al[1] = xi * e1 * e3; al[2] = xi * (1. - e1 * e2); al[3] = xi * e1 * (1. - e2);
            return pow(xi, 3) * (e1 * e1);
        case 1: al[0] = xi; al[1] = xi * e1; al[2] = xi * (1. - e1 * e2 * e3); al[3] = xi * e1 * e2 * (1. - e3); break;
        case 2: al[0] = xi * (1. - e1 * e2); al[1] = xi * e1 * (1. - e2); al[2] = xi; al[3] = xi * e1 * e2 * e3; break;
        case 3: al[0] = xi * (1. - e1 * e2 * e3); al[1] = xi * e1 * e2 * (1. - e3); al[2] = xi; al[3] = xi * e1; break;
        default: al[0] = xi * (1. - e1 * e2 * e3); al[1] = xi * e1 * (1. - e2 * e3); al[2] = xi; al[3] = xi * e1 * e2; break;
        }
        return pow(xi, 3) * (e1 * e1) * e2;
    }
    switch (t) {
    case 0: al[0] = xi; al[1] = xi * (1. - e1 + e1 * e2); al[2] = xi * (1. - e1 * e2 * e3); al[3] = xi * (1. - e1); break;
    case 1: al[0] = xi * (1. - e1 * e2 * e3); al[1] = xi * (1. - e1); al[2] = xi; al[3] = xi * (1. - e1 + e1 * e2); break;
    case 2: al[0] = xi; al[1] = xi * e1 * (1. - e2 + e2 * e3); al[2] = xi * (1. - e1 * e2); al[3] = xi * e1 * (1. - e2); break;
    case 3: al[0] = xi * (1. - e1 * e2); al[1] = xi * e1 * (1. - e2); al[2] = xi; al[3] = xi * e1 * (1. - e2 + e2 * e3); break;
    case 4: al[0] = xi * (1. - e1 * e2 * e3); al[1] = xi * e1 * (1. - e2 * e3); al[2] = xi; al[3] = xi * e1 * (1. - e2); break;
    default: al[0] = xi; al[1] = xi * e1 * (1. - e2); al[2] = xi * (1. - e1 * e2 * e3); al[3] = xi * e1 * (1. - e2 * e3); break;
    }
    return pow(xi, 3) * (e1 * e1) * e2;
}

// ---------------------------------------------------------------- session
// How the quadrature pass adds into the matrix: colored two-sided passes (FP64, and mixed rules
// without a one-sided kernel), or one persistent one-sided pass with fixed-point atomics.
enum { PM_COLORED = 0, PM_RETRI = 1, PM_BARY = 2, PM_VEC = 3 };

struct Session {
    int dim = 2, dV = 3, nProb = 0;
    bool system = true;
    long long nE = 0, nV = 0;
    int maxNE = 0, maxNV = 0;
    int nSM = 148;
    std::vector<ProbParams> hprm;
    std::vector<int> eoff, voff;   // nProb + 1
    Rule rule;
    int duffy_nPg = 0;
    cudaStream_t st = nullptr;
    cudaEvent_t ev[8];
    // inputs
    DevBuf T64, labT64, V, labV64, eoffd, voffd, prm, duffy;
    DevBuf duffyf;   // FP32 Duffy tables of the mixed close-pair rule: points (float4), weights
    // derived
    DevBuf T32, labT, eprob, EC, adet, labV, vprob, EChi, EClo, adetf;
    DevBuf BCf;   // element barycenters as double-float pairs (BC_STRIDE floats per element)
    DevBuf color, color2, colorlist, closeA, closeB, closebuf, touched;
    std::vector<int> color_off;
    int prec = 0;
    bool onesided64 = false;   // PM_RETRI pass in FP64 (the mixed path's algorithm, FP64 arithmetic)
    DevBuf vcnt, vptr, vel, adjcnt, xadj, adj;
    DevBuf stamp_epoch;   // per-warp stamp epochs of the search
    long long stamp_layout[3] = {0, 0, 0};   // warps, element and vertex stride the stamps were laid out for
    DevBuf visited, vvisited, queue, pool, seg_start, seg_cnt, out_ptr, pA, pB, incnt, in_ptr, inA;
    DevBuf marks, rowcnt, rowptr, cols, acc, tiny, vals, keepcnt, fptr, fcols, fvals;
    DevBuf closelist, scan_tmp, counters, err, facc, ftiny, fd;
    DevBuf out64a, out64b;
    DevBuf hcap, hptr, htab, tpos, dslot;   // slot maps of the one-sided passes
    DevBuf rwords, rbase, rlo, rankmap;      // window-rank slot map (slots.cuh)
    // one-sided passes: per element, the vertices of its partners and its own (row patterns)
    DevBuf eid_ptr, eid, vp_cnt, vp_off, vp_ptr, vp_scratch;
    long long vp_cap = 0;
    bool vlists = false;
    bool use_rank = false;
    bool pairs_pool = false;        // out-lists are the search's pool segments (run_pairs)
    bool want_pair_arrays = false;  // the pair-list hook asks for aT-major pA / pB
    long long rtot = 0;
    DevBuf pscratch, rowoff;                // single-pass pattern (capacity from the last assembly)
    DevBuf valsN, elp;                      // one-sided retriangulate pass: own-row termNonloc, LP blocks
    DevBuf po_cnt, po_off, po_ptr, po_scratch, tcnt, tptr, tcols;   // transposed pattern construction
    long long po_cap = 0, t_nnz = 0;
    DevBuf sv_vec, sv_part;                 // CG solve: f, g, b, x, r, p, Ap; dot partials
    DevBuf zptr, zidx;                      // domain-decomposition indicator (element -> subdomains)
    DevBuf vacc, vtiny;                     // vector path: 128-bit sums per expanded slot
    DevBuf kclist;                          // elements grouped by kernel class (pass launches)
    // Discontinuous Galerkin: after the pair search, dg_swap_in swaps the row space to the element
    // DOFs dV e + a (the identity table, every row kept, K = dV nE rows). T32, labV, vprob, vptr,
    // vel, nV, maxNV and voff then describe DOF rows for the pattern, the passes, the finish and
    // the download; the next run_prep swaps the mesh's vertices back (dg_restore).
    bool dg = false, dg_rows = false;
    long long dg_saved_nV = 0;
    int dg_saved_maxNV = 0, dg_saved_pnV = 0;
    DevBuf dgT32, dglabV, dgvprob, dgvptr, dgvel;
    long long kc_off[4] = {-1, 0, 0, 0};    // class offsets into kclist (-1: list not built)
    long long pat_cap = 0;
    // one-shot calls: the previous call's pattern size, used as the scratch capacity when the
    // mesh has the same element and vertex counts (an overflow falls back to two passes)
    long long hint_pat_cap = 0, hint_po_cap = 0, hint_vp_cap = 0, hint_nE = -1, hint_nV = -1;
    int pmode = 0;                          // PM_COLORED, PM_RETRI, PM_BARY or PM_VEC
    int od = 1;                             // outdim: rows od v + i (PM_VEC when od > 1)
    int tune_bfs = 0, tune_pass = 0;        // blocks per SM of the search / persistent pass (0: occupancy)
    int used_bfs = 0, used_pass = 0;        // what the last assembly launched
    // graph replay: the stages run without host reads, on the sizes of the previous assembly
    bool replay = false;
    long long nadj = 0, htot = 0;
    cudaGraphExec_t gexec = nullptr;
    long long qcap = 0, pool_cap = 0;
    long long P = 0, nnz_struct = 0, nnz = 0;
    long long nlaunch = 0;   // kernels launched by the current assembly
    nlfem_stats stats;
    // every device buffer of the session, in a fixed order
    std::vector<DevBuf *> buffers() {
        return {&T64, &labT64, &V, &labV64, &eoffd, &voffd, &prm, &duffy, &duffyf, &T32, &labT, &eprob,
                &EC, &adet, &labV, &vprob, &vcnt, &vptr, &vel, &adjcnt, &xadj, &adj, &visited, &vvisited, &stamp_epoch,
                &queue, &pool, &seg_start, &seg_cnt, &out_ptr, &pA, &pB, &incnt, &in_ptr, &inA,
                &marks, &rowcnt, &rowptr, &cols, &acc, &tiny, &vals, &keepcnt, &fptr, &fcols,
                &fvals, &closelist, &scan_tmp, &counters, &err, &facc, &ftiny, &fd, &out64a, &out64b,
                &EChi, &EClo, &adetf, &BCf, &color, &color2, &colorlist, &closeA, &closeB, &closebuf, &touched,
                &hcap, &hptr, &htab, &tpos, &dslot, &rwords, &rbase, &rlo, &rankmap, &eid_ptr, &eid, &vp_cnt, &vp_off, &vp_ptr, &vp_scratch, &pscratch, &rowoff, &kclist, &valsN, &elp,
                &po_cnt, &po_off, &po_ptr, &po_scratch, &tcnt, &tptr, &tcols, &sv_vec, &sv_part, &zptr, &zidx, &vacc, &vtiny,
                &dgT32, &dglabV, &dgvprob, &dgvptr, &dgvel};
    }
    ~Session() {
        for (DevBuf *b : buffers()) b->release();
        if (gexec) cudaGraphExecDestroy(gexec);
        if (st) {
            for (int i = 0; i < 8; i++) cudaEventDestroy(ev[i]);
            cudaStreamDestroy(st);
        }
    }
};

// Exclusive scan of n inputs into n+1 outputs (out[n] = total), int64 results.
template <typename TIn>
static int scan_excl(Session &S, const TIn *in, long long n, long long *out) {
    const long long n_out = n + 1;
    std::vector<long long> sizes;
    long long m = n_out;
    // recursion over block sums kept in scan_tmp
    long long nb = (m + SCAN_TILE - 1) / SCAN_TILE;
    long long total_tmp = 0, t = nb;
    while (true) {
        total_tmp += 2 * t + 2;
        if (t <= 1) break;
        t = (t + SCAN_TILE - 1) / SCAN_TILE;
    }
    ENS(S.scan_tmp, (size_t)total_tmp * sizeof(long long));
    long long *tmp = S.scan_tmp.get<long long>();
    // level 0
    struct Lvl { long long n; long long *bsum; long long *boff; long long nb; };
    std::vector<Lvl> lv;
    lv.push_back({m, tmp, tmp + nb + 1, nb});
    k_scan_reduce<TIn><<<(unsigned)nb, SCAN_THREADS, 0, S.st>>>(in, n, lv[0].bsum); ++S.nlaunch;
    long long off = 2 * nb + 2;
    while (lv.back().nb > 1) {
        Lvl &pl = lv.back();
        long long nb2 = (pl.nb + SCAN_TILE - 1) / SCAN_TILE;
        Lvl l2{pl.nb, tmp + off, tmp + off + nb2 + 1, nb2};
        off += 2 * nb2 + 2;
        k_scan_reduce<long long><<<(unsigned)nb2, SCAN_THREADS, 0, S.st>>>(pl.bsum, pl.nb, l2.bsum); ++S.nlaunch;
        lv.push_back(l2);
    }
    // top level: single block sum -> offset 0
    CK(cudaMemsetAsync(lv.back().boff, 0, sizeof(long long), S.st));
    for (int i = (int)lv.size() - 1; i >= 1; i--) {
        // scan level i-1 block sums using level i offsets
        k_scan_down<long long><<<(unsigned)lv[i].nb, SCAN_THREADS, 0, S.st>>>(lv[i - 1].bsum, lv[i - 1].nb, lv[i - 1].nb, lv[i].boff, lv[i - 1].boff); ++S.nlaunch;
    }
    // final: scan n inputs (+1 trailing zero) into out
    (void)sizes;
    k_scan_down<TIn><<<(unsigned)nb, SCAN_THREADS, 0, S.st>>>(in, n, n_out, lv[0].boff, out); ++S.nlaunch;
    CK(cudaGetLastError());
    return NLFEM_OK;
}

template <typename T>
static int d2h(Session &S, T *host, const T *dev, size_t n) {
    if (S.replay) return NLFEM_OK;   // captured sequence: the host values are those of the last run
    CK(cudaMemcpyAsync(host, dev, n * sizeof(T), cudaMemcpyDeviceToHost, S.st));
    CK(cudaStreamSynchronize(S.st));
    return NLFEM_OK;
}

static int device_ok();

// Host checks of the problems first (they need no device, so a configuration error is reported as
// such on any machine), then the device: stream, events, uploads.
static int session_init(Session &S, const nlfem_problem *probs, int n, bool system) {
    S.system = system;
    S.nProb = n;
    S.dim = probs[0].dim;
    S.dV = S.dim + 1;
    S.hprm.resize(n);
    S.eoff.assign(n + 1, 0);
    S.voff.assign(n + 1, 0);
    for (int i = 0; i < n; i++) {
        const nlfem_problem &p = probs[i];
        if (p.dim != S.dim) return fail(NLFEM_ERR_INVALID, "all problems of a batch must share the dimension");
        int r = make_params(p, system, S.hprm[i]);
        if (r) return r;
        S.hprm[i].elem_off = (int)S.eoff[i];
        S.hprm[i].vert_off = (int)S.voff[i];
        S.hprm[i].nE = (int)p.nE;
        S.hprm[i].nV = (int)p.nV;
        if ((long long)S.eoff[i] + p.nE >= (1LL << 31) || (long long)S.voff[i] + p.nV >= (1LL << 31))
            return fail(NLFEM_ERR_UNSUPPORTED, "batch too large (2^31 elements or vertices)");
        S.eoff[i + 1] = S.eoff[i] + (int)p.nE;
        S.voff[i + 1] = S.voff[i] + (int)p.nV;
        S.maxNE = std::max(S.maxNE, (int)p.nE);
        S.maxNV = std::max(S.maxNV, (int)p.nV);
    }
    S.nE = S.eoff[n];
    S.nV = S.voff[n];
    S.dg = probs[0].is_dg != 0;
    S.dg_rows = false;
    for (int i = 1; i < n; i++)
        if ((probs[i].is_dg != 0) != S.dg) return fail(NLFEM_ERR_UNSUPPORTED, "all problems of a batch must share the ansatz");
    if (S.dg && n > 1) return fail(NLFEM_ERR_UNSUPPORTED, "DG problems assemble one at a time (no batches)");
    S.prec = probs[0].precision == NLFEM_PREC_MIXED ? PREC_MIX : PREC_F64;
    S.onesided64 = probs[0].precision == NLFEM_PREC_FP64_ONESIDED;
    for (int i = 1; i < n; i++)
        if (probs[i].precision != probs[0].precision)
            return fail(NLFEM_ERR_UNSUPPORTED, "all problems of a batch must share the precision");
    S.od = probs[0].outdim;
    for (int i = 1; i < n; i++)
        if (probs[i].outdim != S.od) return fail(NLFEM_ERR_UNSUPPORTED, "all problems of a batch must share the outdim");
    int r = make_rule(probs[0], system, S.rule);
    if (r) return r;
    for (int i = 1; i < n; i++) {
        Rule r2;
        int rr = make_rule(probs[i], system, r2);
        if (rr) return rr;
        if (memcmp(&r2, &S.rule, sizeof(Rule)) != 0)
            return fail(NLFEM_ERR_UNSUPPORTED, "all problems of a batch must share the quadrature rules");
    }
    {
        // one-sided fixed-point passes for the mixed precision; colored passes otherwise
        bool all_retri = system, all_bary = system, any_singular = false, any_zeta = false;
        for (const ProbParams &q : S.hprm) {
            all_retri &= (q.remote == MTH_RETRIANGULATE);
            all_bary &= (q.remote == MTH_BARYCENTER);
            any_singular |= q.singular != 0;
            any_zeta |= q.zeta != 0;
        }
        // domain-decomposition weights run in the colored passes (either precision)
        S.pmode = PM_COLORED;
        if (S.prec == PREC_MIX && S.dim == 2 && all_retri && !any_zeta) S.pmode = PM_RETRI;
        if (S.prec == PREC_MIX && all_bary && !any_singular && !any_zeta) S.pmode = PM_BARY;
        if (S.od > 1) S.pmode = PM_VEC;
        if (S.onesided64) {
            if (!(S.dim == 2 && all_retri && !any_zeta))
                return fail(NLFEM_ERR_UNSUPPORTED, "precision \"fp64-onesided\" covers the 2D retriangulate rule "
                                                   "without domain-decomposition weights");
            S.pmode = PM_RETRI;
        }
    }
    r = device_ok();
    if (r) return r;
    {
        int dev = 0;
        CK(cudaGetDevice(&dev));
        CK(cudaDeviceGetAttribute(&S.nSM, cudaDevAttrMultiProcessorCount, dev));
        CK(cudaStreamCreateWithFlags(&S.st, cudaStreamNonBlocking));
        for (int i = 0; i < 8; i++) CK(cudaEventCreate(&S.ev[i]));
    }
    const int dV = S.dV, dim = S.dim;
    ENS(S.T64, sizeof(long long) * S.nE * dV);
    ENS(S.labT64, sizeof(long long) * S.nE);
    ENS(S.V, sizeof(double) * S.nV * dim);
    ENS(S.labV64, sizeof(long long) * S.nV);
    ENS(S.eoffd, sizeof(int) * (n + 1));
    ENS(S.voffd, sizeof(int) * (n + 1));
    ENS(S.prm, sizeof(ProbParams) * n);
    CK(cudaMemcpyAsync(S.eoffd.p, S.eoff.data(), sizeof(int) * (n + 1), cudaMemcpyHostToDevice, S.st));
    CK(cudaMemcpyAsync(S.voffd.p, S.voff.data(), sizeof(int) * (n + 1), cudaMemcpyHostToDevice, S.st));
    CK(cudaMemcpyAsync(S.prm.p, S.hprm.data(), sizeof(ProbParams) * n, cudaMemcpyHostToDevice, S.st));
    // Duffy tables (shared by the batch's singular problems: same tensor degree and s required)
    if (system) {
        int first = -1;
        for (int i = 0; i < n; i++)
            if (duffy_close(S.hprm[i]) && first < 0) first = i;
        if (first >= 0) {
            const nlfem_problem &p = probs[first];
            const int deg = p.tensorGaussDegree;
            const int nPg = deg * deg * deg * deg;
            for (int i = first + 1; i < n; i++)
                if (duffy_close(S.hprm[i]) &&
                    (probs[i].tensorGaussDegree != deg || probs[i].fractional_s != p.fractional_s))
                    return fail(NLFEM_ERR_UNSUPPORTED, "batched singular problems must share degree and s");
            S.duffy_nPg = nPg;
            const int nTr[3] = {2, 5, 6};
            std::vector<double> h;
            for (int c = 0; c < 3; c++) {
                std::vector<double> al((size_t)nTr[c] * nPg * 4), td((size_t)nTr[c] * nPg);
                std::vector<double> au((size_t)nTr[c] * nPg * 4), tw((size_t)nTr[c] * nPg);
                for (int t = 0; t < nTr[c]; t++)
                    for (int k = 0; k < nPg; k++) {
                        double *a = &al[((size_t)t * nPg + k) * 4], *u = &au[((size_t)t * nPg + k) * 4];
                        for (int j = 0; j < 4; j++) a[j] = p.Pg[4 * k + j] * 0.5 + 0.5;
                        for (int j = 0; j < 4; j++) u[j] = a[j];
                        double tdf = pow(a[0], 3 - 2 * p.fractional_s);
                        double tdw = pow(a[0], 3 - 2 - 2 * p.fractional_s);   // weakSingular
                        a[0] = 1.0;
                        duffy_traffo(c, t, u);
                        double det = duffy_traffo(c, t, a);
                        tdf *= det * 0.0625;
                        tdw *= det * 0.0625;
                        a[0] = a[0] - a[1];
                        a[2] = a[2] - a[3];
                        u[0] = u[0] - u[1];
                        u[2] = u[2] - u[3];
                        td[(size_t)t * nPg + k] = tdf;
                        tw[(size_t)t * nPg + k] = tdw;
                    }
                h.insert(h.end(), al.begin(), al.end());
                h.insert(h.end(), td.begin(), td.end());
                h.insert(h.end(), au.begin(), au.end());
                h.insert(h.end(), tw.begin(), tw.end());
            }
            h.insert(h.end(), p.dg, p.dg + nPg);
            ENS(S.duffy, sizeof(double) * h.size());
            CK(cudaMemcpyAsync(S.duffy.p, h.data(), sizeof(double) * h.size(), cudaMemcpyHostToDevice, S.st));
            // FP32 copies for the mixed path: per case the points and the weights tdet * dg
            std::vector<float> hf;
            {
                size_t o = 0;
                const double *dg = &h[h.size() - nPg];
                for (int c = 0; c < 3; c++) {
                    const size_t np = (size_t)nTr[c] * nPg;
                    for (size_t i = 0; i < np * 4; i++) hf.push_back((float)h[o + i]);
                    for (size_t i = 0; i < np; i++) hf.push_back((float)(h[o + np * 4 + i] * dg[i % nPg]));
                    while (hf.size() % 4) hf.push_back(0.f);   // the next float4 points stay 16-byte aligned
                    for (size_t i = 0; i < np * 4; i++) hf.push_back((float)h[o + np * 5 + i]);   // alphaU
                    for (size_t i = 0; i < np; i++) hf.push_back((float)(h[o + np * 9 + i] * dg[i % nPg]));   // tdetW dg
                    while (hf.size() % 4) hf.push_back(0.f);
                    o += np * 4 + np + np * 4 + np;
                }
            }
            ENS(S.duffyf, sizeof(float) * hf.size());
            CK(cudaMemcpyAsync(S.duffyf.p, hf.data(), sizeof(float) * hf.size(), cudaMemcpyHostToDevice, S.st));
            CK(cudaStreamSynchronize(S.st));
        }
    }
    return NLFEM_OK;
}

// Host -> device copy of the meshes (the per-step input traffic of the end-to-end path).
static int session_upload(Session &S, const nlfem_problem *probs) {
    const int dV = S.dV, dim = S.dim;
    bool any_zeta = false;
    for (int i = 0; i < S.nProb; i++) any_zeta = any_zeta || S.hprm[i].zeta;
    if (any_zeta) {   // one indicator CSR over the batch's elements (problems without: empty rows)
        std::vector<long long> zp((size_t)S.nE + 1, 0), zi;
        for (int i = 0; i < S.nProb; i++) {
            const nlfem_problem &p = probs[i];
            for (long e = 0; e < p.nE; e++) {
                if (S.hprm[i].zeta)
                    for (long k = p.zeta_indptr[e]; k < p.zeta_indptr[e + 1]; k++) zi.push_back(p.zeta_indices[k]);
                zp[(size_t)S.eoff[i] + e + 1] = (long long)zi.size();
            }
        }
        ENS(S.zptr, sizeof(long long) * zp.size());
        ENS(S.zidx, sizeof(long long) * (zi.size() + 1));
        CK(cudaMemcpyAsync(S.zptr.p, zp.data(), sizeof(long long) * zp.size(), cudaMemcpyHostToDevice, S.st));
        if (!zi.empty()) CK(cudaMemcpyAsync(S.zidx.p, zi.data(), sizeof(long long) * zi.size(), cudaMemcpyHostToDevice, S.st));
        CK(cudaStreamSynchronize(S.st));   // the host vectors go out of scope
    }
    for (int i = 0; i < S.nProb; i++) {
        const nlfem_problem &p = probs[i];
        CK(cudaMemcpyAsync(S.T64.get<long long>() + (long long)S.eoff[i] * dV, p.elements, sizeof(long long) * p.nE * dV, cudaMemcpyHostToDevice, S.st));
        CK(cudaMemcpyAsync(S.labT64.get<long long>() + S.eoff[i], p.elementLabels, sizeof(long long) * p.nE, cudaMemcpyHostToDevice, S.st));
        CK(cudaMemcpyAsync(S.V.get<double>() + (long long)S.voff[i] * dim, p.vertices, sizeof(double) * p.nV * dim, cudaMemcpyHostToDevice, S.st));
        CK(cudaMemcpyAsync(S.labV64.get<long long>() + S.voff[i], p.vertexLabels, sizeof(long long) * p.nV, cudaMemcpyHostToDevice, S.st));
    }
    return NLFEM_OK;
}

__global__ void k_dg_rows(long long K, int dV, int *__restrict__ T32, int *__restrict__ labV, int *__restrict__ vprob,
                          long long *__restrict__ vptr, int *__restrict__ vel) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i > K) return;
    vptr[i] = i;
    if (i == K) return;
    T32[i] = (int)i;   // element e, local vertex a -> DOF dV e + a
    labV[i] = 1;       // every DG row is kept (Cassemble.cpp:735, 751)
    vprob[i] = 0;
    vel[i] = (int)(i / dV);
}

// Row space of a DG assembly (one problem): the element DOFs.
static int dg_swap_in(Session &S) {
    const long long K = (long long)S.dV * S.nE;
    ENS(S.dgT32, sizeof(int) * (K + 1));
    ENS(S.dglabV, sizeof(int) * (K + 1));
    ENS(S.dgvprob, sizeof(int) * (K + 1));
    ENS(S.dgvptr, sizeof(long long) * (K + 1));
    ENS(S.dgvel, sizeof(int) * (K + 1));
    k_dg_rows<<<grid_for(K + 1, 256), 256, 0, S.st>>>(K, S.dV, S.dgT32.get<int>(), S.dglabV.get<int>(), S.dgvprob.get<int>(),
                                                      S.dgvptr.get<long long>(), S.dgvel.get<int>()); ++S.nlaunch;
    CK(cudaGetLastError());
    std::swap(S.T32, S.dgT32); std::swap(S.labV, S.dglabV); std::swap(S.vprob, S.dgvprob);
    std::swap(S.vptr, S.dgvptr); std::swap(S.vel, S.dgvel);
    S.dg_saved_nV = S.nV; S.dg_saved_maxNV = S.maxNV; S.dg_saved_pnV = S.hprm[0].nV;
    S.nV = K; S.maxNV = (int)K; S.voff[1] = (int)K; S.hprm[0].nV = (int)K;
    CK(cudaMemcpyAsync(S.prm.p, S.hprm.data(), sizeof(ProbParams), cudaMemcpyHostToDevice, S.st));
    CK(cudaMemcpyAsync(S.voffd.p, S.voff.data(), sizeof(int) * 2, cudaMemcpyHostToDevice, S.st));
    S.dg_rows = true;
    return NLFEM_OK;
}

static int dg_restore(Session &S) {
    if (!S.dg_rows) return NLFEM_OK;
    std::swap(S.T32, S.dgT32); std::swap(S.labV, S.dglabV); std::swap(S.vprob, S.dgvprob);
    std::swap(S.vptr, S.dgvptr); std::swap(S.vel, S.dgvel);
    S.nV = S.dg_saved_nV; S.maxNV = S.dg_saved_maxNV; S.voff[1] = (int)S.dg_saved_nV; S.hprm[0].nV = S.dg_saved_pnV;
    CK(cudaMemcpyAsync(S.prm.p, S.hprm.data(), sizeof(ProbParams), cudaMemcpyHostToDevice, S.st));
    CK(cudaMemcpyAsync(S.voffd.p, S.voff.data(), sizeof(int) * 2, cudaMemcpyHostToDevice, S.st));
    S.dg_rows = false;
    return NLFEM_OK;
}

template <int DIM>
static int run_prep(Session &S) {
    int rr = dg_restore(S);
    if (rr) return rr;
    const long long nE = S.nE, nV = S.nV;
    constexpr int dV = DIM + 1;
    ENS(S.T32, sizeof(int) * nE * dV);
    ENS(S.labT, sizeof(int) * nE);
    ENS(S.eprob, sizeof(int) * nE);
    ENS(S.EC, sizeof(double) * nE * DIM * dV);
    ENS(S.adet, sizeof(double) * nE);
    ENS(S.EChi, sizeof(float) * nE * DIM * dV);
    ENS(S.adetf, sizeof(float) * nE);
    ENS(S.EClo, sizeof(float) * nE * DIM * dV);
    ENS(S.BCf, sizeof(float) * nE * BC_STRIDE<DIM>);
    ENS(S.labV, sizeof(int) * nV);
    ENS(S.vprob, sizeof(int) * nV);
    ENS(S.counters, sizeof(unsigned long long) * 16);
    ENS(S.err, sizeof(int) * 16);
    CK(cudaMemsetAsync(S.counters.p, 0, sizeof(unsigned long long) * 16, S.st));
    CK(cudaMemsetAsync(S.err.p, 0, sizeof(int) * 16, S.st));
    k_prep_elements<DIM><<<grid_for(nE, 256), 256, 0, S.st>>>(
        S.T64.get<long long>(), S.labT64.get<long long>(), S.V.get<double>(), S.eoffd.get<int>(),
        S.voffd.get<int>(), S.nProb, nE, S.T32.get<int>(), S.labT.get<int>(), S.eprob.get<int>(),
        S.EC.get<double>(), S.adet.get<double>(), S.EChi.get<float>(), S.EClo.get<float>(), S.adetf.get<float>(), S.BCf.get<float>()); ++S.nlaunch;
    k_prep_vertices<<<grid_for(nV, 256), 256, 0, S.st>>>(S.labV64.get<long long>(), S.voffd.get<int>(),
        S.nProb, nV, S.labV.get<int>(), S.vprob.get<int>()); ++S.nlaunch;
    CK(cudaGetLastError());
    return NLFEM_OK;
}

template <int DIM>
static int run_dual(Session &S) {
    constexpr int dV = DIM + 1;
    const long long nE = S.nE, nV = S.nV;
    ENS(S.vcnt, sizeof(int) * (nV + 1));
    ENS(S.vptr, sizeof(long long) * (nV + 1));
    ENS(S.vel, sizeof(int) * nE * dV);
    CK(cudaMemsetAsync(S.vcnt.p, 0, sizeof(int) * (nV + 1), S.st));
    k_vinc_count<<<grid_for(nE * dV, 256), 256, 0, S.st>>>(S.T32.get<int>(), nE * dV, S.vcnt.get<int>()); ++S.nlaunch;
    int r = scan_excl<int>(S, S.vcnt.get<int>(), nV, S.vptr.get<long long>());
    if (r) return r;
    CK(cudaMemsetAsync(S.vcnt.p, 0, sizeof(int) * (nV + 1), S.st));
    k_vinc_fill<<<grid_for(nE * dV, 256), 256, 0, S.st>>>(S.T32.get<int>(), nE * dV, dV, S.vptr.get<long long>(), S.vcnt.get<int>(), S.vel.get<int>()); ++S.nlaunch;
    k_vinc_sort<<<grid_for(nV, 256), 256, 0, S.st>>>(S.vptr.get<long long>(), nV, S.vel.get<int>()); ++S.nlaunch;
    // The search walks the vertex incidence lists. The element dual graph is needed only by the
    // element coloring of the colored passes and by the close-pair slots of singular kernels.
    bool need_adj = S.pmode == PM_COLORED;
    for (const ProbParams &q : S.hprm) need_adj = need_adj || duffy_close(q);
    if (!need_adj) {
        S.nadj = 0;
        CK(cudaGetLastError());
        return NLFEM_OK;
    }
    ENS(S.adjcnt, sizeof(int) * (nE + 1));
    ENS(S.xadj, sizeof(long long) * (nE + 1));
    k_adjacency<DIM><<<grid_for(nE, 128), 128, 0, S.st>>>(S.T32.get<int>(), nE, S.vptr.get<long long>(), S.vel.get<int>(), nullptr, S.adjcnt.get<int>(), nullptr, S.err.get<int>() + 8); ++S.nlaunch;
    r = scan_excl<int>(S, S.adjcnt.get<int>(), nE, S.xadj.get<long long>());
    if (r) return r;
    r = d2h(S, &S.nadj, S.xadj.get<long long>() + nE, 1);
    if (r) return r;
    ENS(S.adj, sizeof(int) * (S.nadj + 1));
    k_adjacency<DIM><<<grid_for(nE, 128), 128, 0, S.st>>>(S.T32.get<int>(), nE, S.vptr.get<long long>(), S.vel.get<int>(), S.xadj.get<long long>(), S.adjcnt.get<int>(), S.adj.get<int>(), S.err.get<int>() + 8); ++S.nlaunch;
    CK(cudaGetLastError());
    if (S.replay) return NLFEM_OK;
    int e8 = 0;
    r = d2h(S, &e8, S.err.get<int>() + 8, 1);
    if (r) return r;
    if (e8) return fail(NLFEM_ERR_UNSUPPORTED, "element with more than 320 vertex neighbours");
    return NLFEM_OK;
}

template <int DIM>
static int run_bfs(Session &S) {
    const long long nE = S.nE;
    // visited set: per-warp stamp arrays in global memory. (A shared-memory bitmap over the
    // problem's elements was measured slower: neighbouring candidates share a word, so the
    // shared-memory atomics serialise, and the bitmaps cap the occupancy.)
    auto kfn = S.prec == PREC_MIX ? k_bfs<DIM, PREC_MIX> : k_bfs<DIM, PREC_F64>;
    int per_sm = 0;
    CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kfn, BFS_THREADS, 0));
    per_sm = std::max(per_sm, 1);
    if (S.tune_bfs > 0) per_sm = std::min(per_sm, S.tune_bfs);   // autotuned (nlfem_session_autotune)
    S.used_bfs = per_sm;
    const int nblocks = S.nSM * per_sm;
    const int nwarps = nblocks * BFS_WARPS;
    if (S.qcap == 0) S.qcap = std::min<long long>(S.maxNE + 1, 8192);
    if (S.pool_cap == 0) {
        // expected pairs: per outer element, the elements meeting a ball of radius delta + 2h
        // (h the mean element size), with 10% headroom; a short pool only costs a retry
        double est = 0;
        for (const ProbParams &q : S.hprm) {
            const double h = S.dim == 2 ? sqrt(2.0 * q.el) : cbrt(6.0 * q.el);
            const double r = q.delta + 2.0 * h;
            const double ball = S.dim == 2 ? M_PI * r * r : 4.0 / 3.0 * M_PI * r * r * r;
            est += (double)q.nE * std::min((double)q.nE, ball / std::max(q.el, 1e-300) + 16.0);
        }
        S.pool_cap = std::max<long long>((long long)(1.1 * est), 1 << 20);
    }
    {   // stamps: zeroed only when first laid out (a new layout or a larger buffer)
        const size_t be = sizeof(unsigned short) * (size_t)nwarps * S.maxNE;
        const size_t bv = sizeof(unsigned short) * (size_t)nwarps * S.maxNV;
        const size_t bw = sizeof(unsigned) * (size_t)nwarps;
        const bool relayout = be > S.visited.cap || bv > S.vvisited.cap || bw > S.stamp_epoch.cap ||
                              S.stamp_layout[0] != nwarps || S.stamp_layout[1] != S.maxNE ||
                              S.stamp_layout[2] != S.maxNV;
        ENS(S.visited, be);
        ENS(S.vvisited, bv);
        ENS(S.stamp_epoch, bw);
        if (relayout) {
            CK(cudaMemsetAsync(S.visited.p, 0, be, S.st));
            CK(cudaMemsetAsync(S.vvisited.p, 0, bv, S.st));
            CK(cudaMemsetAsync(S.stamp_epoch.p, 0, bw, S.st));
            S.stamp_layout[0] = nwarps;
            S.stamp_layout[1] = S.maxNE;
            S.stamp_layout[2] = S.maxNV;
        }
    }
    ENS(S.seg_start, sizeof(long long) * (nE + 1));
    ENS(S.seg_cnt, sizeof(int) * (nE + 1));
    for (int attempt = 0; attempt < 8; attempt++) {
        ENS(S.queue, sizeof(int) * (size_t)nwarps * S.qcap);
        ENS(S.pool, sizeof(int) * (size_t)S.pool_cap);
        CK(cudaMemsetAsync(S.counters.p, 0, sizeof(unsigned long long) * 8, S.st));
        CK(cudaMemsetAsync(S.err.p, 0, sizeof(int) * 4, S.st));
        BfsArgs a;
        memset(&a, 0, sizeof(a));
        a.T32 = S.T32.get<int>(); a.labT = S.labT.get<int>(); a.eprob = S.eprob.get<int>();
        a.EC = S.EC.get<double>();
        a.EChi = S.EChi.get<float>(); a.EClo = S.EClo.get<float>(); a.BCf = S.BCf.get<float>();
        a.probs = S.prm.get<ProbParams>(); a.nE = nE;
        a.visited = S.visited.get<unsigned short>(); a.vstride = S.maxNE;
        a.epoch = S.stamp_epoch.get<unsigned>();
        a.vptr = S.vptr.get<long long>(); a.vel = S.vel.get<int>();
        a.vvisited = S.vvisited.get<unsigned short>(); a.vvstride = S.maxNV;
        a.queue = S.queue.get<int>(); a.qcap = S.qcap;
        a.pool = S.pool.get<int>(); a.pool_cap = S.pool_cap;
        unsigned long long *cnt = S.counters.get<unsigned long long>();
        a.pool_cursor = cnt + 0; a.n_cand = cnt + 1; a.qneed = (long long *)(cnt + 2);
        a.seg_start = S.seg_start.get<long long>(); a.seg_cnt = S.seg_cnt.get<int>();
        a.err = S.err.get<int>();
        a.n_amb = cnt + 7;
        a.work = cnt + 3;
        kfn<<<nblocks, BFS_THREADS, 0, S.st>>>(a, S.rule);
        ++S.nlaunch;
        CK(cudaGetLastError());
        if (S.replay) return NLFEM_OK;   // overflow flags are checked after the replay
        unsigned long long hc[3];
        int he[2];
        int r = d2h(S, hc, cnt, 3);
        if (r) return r;
        r = d2h(S, he, S.err.get<int>(), 2);
        if (r) return r;
        if (he[0]) { S.qcap = std::max<long long>((long long)hc[2] * 3 / 2, S.qcap * 2); continue; }
        if (he[1]) { S.pool_cap = (long long)hc[0] + (long long)hc[0] / 8 + 1024; continue; }
        S.stats.n_candidates = (long)hc[1];
        return NLFEM_OK;
    }
    return fail(NLFEM_ERR_NOMEM, "BFS capacity retries exhausted");
}

static int sort_segments(Session &S, const long long *ptr, long long nseg, int *data) {
    const int cap = 16384;
    CK(cudaFuncSetAttribute(k_row_sort, cudaFuncAttributeMaxDynamicSharedMemorySize, cap * (int)sizeof(int)));
    k_row_sort<<<S.nSM * 4, 256, cap * sizeof(int), S.st>>>(ptr, nseg, data, cap); ++S.nlaunch;
    k_row_sort_global<<<S.nSM * 4, 256, 0, S.st>>>(ptr, nseg, data, cap); ++S.nlaunch;
    CK(cudaGetLastError());
    return NLFEM_OK;
}

// Threads per block of the shared-memory bitmap pattern kernel (0: a problem's vertex bitmap is too
// large, the global-memory marks kernel runs instead).
static int pattern_bitmap_threads(const Session &S) {
    const int words = (S.maxNV + 31) / 32;
    if ((size_t)words * 4 * 8 <= 200 * 1024) return 256;
    if ((size_t)words * 4 * 2 <= 200 * 1024) return 64;
    return 0;
}

template <int DIM>
static int run_pairs(Session &S) {
    const long long nE = S.nE;
    // The one-sided passes and their bitmap pattern read each element's partners where the search
    // left them (its segment of the pool: seg_start, seg_cnt), so the pairs are held once (4 B
    // each). The other paths, and the pair-list hook, get aT-major arrays pA, pB and out_ptr.
    S.pairs_pool = !S.want_pair_arrays &&
                   (S.pmode == PM_BARY || S.pmode == PM_RETRI) && pattern_bitmap_threads(S);
    if (S.pairs_pool) {
        int r = d2h(S, &S.P, reinterpret_cast<long long *>(S.counters.get<unsigned long long>()), 1);   // pool cursor
        if (r) return r;
        S.stats.n_pairs = (long)S.P;
        CK(cudaGetLastError());
        return NLFEM_OK;
    }
    ENS(S.out_ptr, sizeof(long long) * (nE + 1));
    int r = scan_excl<int>(S, S.seg_cnt.get<int>(), nE, S.out_ptr.get<long long>());
    if (r) return r;
    r = d2h(S, &S.P, S.out_ptr.get<long long>() + nE, 1);
    if (r) return r;
    const long long P = S.P;
    ENS(S.pA, sizeof(int) * (P + 1));
    ENS(S.pB, sizeof(int) * (P + 1));
    k_compact_pairs<<<grid_for(nE * 32, 256), 256, 0, S.st>>>(S.seg_start.get<long long>(), S.seg_cnt.get<int>(), S.out_ptr.get<long long>(), S.pool.get<int>(), nE, S.pA.get<int>(), S.pB.get<int>()); ++S.nlaunch;
    S.stats.n_pairs = (long)P;
    if (S.pmode == PM_BARY || (S.pmode == PM_RETRI && pattern_bitmap_threads(S))) {
        // barycenter pairs write the outer element's rows only; the retriangulate pattern takes
        // its in-pair columns from the transposed out-pair rows: no in-lists
        CK(cudaGetLastError());
        return NLFEM_OK;
    }
    ENS(S.incnt, sizeof(int) * (nE + 1));
    ENS(S.in_ptr, sizeof(long long) * (nE + 1));
    ENS(S.inA, sizeof(int) * (P + 1));
    CK(cudaMemsetAsync(S.incnt.p, 0, sizeof(int) * (nE + 1), S.st));
    k_in_count<<<grid_for(P, 256), 256, 0, S.st>>>(S.pB.get<int>(), P, S.incnt.get<int>()); ++S.nlaunch;
    r = scan_excl<int>(S, S.incnt.get<int>(), nE, S.in_ptr.get<long long>());
    if (r) return r;
    CK(cudaMemsetAsync(S.incnt.p, 0, sizeof(int) * (nE + 1), S.st));
    k_in_fill<<<grid_for(P, 256), 256, 0, S.st>>>(S.pA.get<int>(), S.pB.get<int>(), P, S.in_ptr.get<long long>(), S.incnt.get<int>(), S.inA.get<int>()); ++S.nlaunch;
    CK(cudaGetLastError());
    // The out-lists come from the BFS in its (deterministic) discovery order. The colored
    // two-sided passes sum the in-lists, which k_in_fill fills in atomic order, so those are
    // sorted; the one-sided pass reads no in-list and the pattern sorts its rows itself.
    if (S.pmode == PM_COLORED) {
        r = sort_segments(S, S.out_ptr.get<long long>(), nE, S.pB.get<int>());
        if (r) return r;
        r = sort_segments(S, S.in_ptr.get<long long>(), nE, S.inA.get<int>());
        if (r) return r;
    }
    S.stats.n_pairs = (long)P;
    return NLFEM_OK;
}

// Deterministic element coloring (Jones-Plassmann rounds, ping-pong buffers) and color lists.
static int run_color(Session &S) {
    const long long nE = S.nE;
    ENS(S.color, sizeof(int) * (nE + 1));
    ENS(S.color2, sizeof(int) * (nE + 1));
    ENS(S.colorlist, sizeof(int) * (nE + 1));
    CK(cudaMemsetAsync(S.color.p, 0xff, sizeof(int) * (nE + 1), S.st));
    unsigned long long *rem = S.counters.get<unsigned long long>() + 8;
    int *cur = S.color.get<int>(), *nxt = S.color2.get<int>();
    for (int round = 0; round < 1000; round++) {
        CK(cudaMemsetAsync(rem, 0, sizeof(unsigned long long), S.st));
        k_color_round<<<grid_for(nE, 256), 256, 0, S.st>>>(S.xadj.get<long long>(), S.adj.get<int>(), nE, S.eprob.get<int>(), S.prm.get<ProbParams>(), cur, nxt, rem, S.err.get<int>() + 9); ++S.nlaunch;
        std::swap(cur, nxt);
        unsigned long long left = 0;
        int r = d2h(S, &left, rem, 1);
        if (r) return r;
        if (left == 0) break;
    }
    if (cur != S.color.get<int>()) CK(cudaMemcpyAsync(S.color.p, cur, sizeof(int) * nE, cudaMemcpyDeviceToDevice, S.st));
    int e9 = 0;
    int r = d2h(S, &e9, S.err.get<int>() + 9, 1);
    if (r) return r;
    if (e9) return fail(NLFEM_ERR_UNSUPPORTED, "more than 256 element colors");
    ENS(S.keepcnt, sizeof(int) * 520);
    int *cnt = S.keepcnt.get<int>();
    CK(cudaMemsetAsync(cnt, 0, sizeof(int) * 520, S.st));
    k_color_count<<<grid_for(nE, 256), 256, 0, S.st>>>(S.color.get<int>(), nE, cnt); ++S.nlaunch;
    std::vector<int> h(256);
    r = d2h(S, h.data(), cnt, 256);
    if (r) return r;
    int nc = 0;
    for (int c = 0; c < 256; c++) if (h[c]) nc = c + 1;
    S.color_off.assign(nc + 1, 0);
    for (int c = 0; c < nc; c++) S.color_off[c + 1] = S.color_off[c] + h[c];
    CK(cudaMemcpyAsync(cnt + 260, S.color_off.data(), sizeof(int) * (nc + 1), cudaMemcpyHostToDevice, S.st));
    CK(cudaMemsetAsync(cnt, 0, sizeof(int) * 256, S.st));
    k_color_fill<<<grid_for(nE, 256), 256, 0, S.st>>>(S.color.get<int>(), nE, cnt + 260, cnt, S.colorlist.get<int>()); ++S.nlaunch;
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(S.st));
    return NLFEM_OK;
}

static SlotMap slot_map(Session &S) {
    SlotMap m;
    m.rowptr = S.rowptr.get<long long>();
    m.hptr = S.hptr.get<long long>();
    m.htab = S.htab.get<unsigned long long>();
    m.rank = S.use_rank ? S.rankmap.get<uint2>() : nullptr;
    m.rbase = S.rbase.get<long long>();
    m.rlo = S.rlo.get<int>();
    m.tpos = S.tpos.get<int>();
    m.dslot = S.dslot.get<int>();
    return m;
}

// Row hash tables, transposed positions and diagonal-block slots (slots.cuh) of the pattern.
template <int DIM>
static int run_slot_maps(Session &S) {
    constexpr int dV = DIM + 1;
    const long long nV = S.nV, nE = S.nE, nnz = S.nnz_struct;
    ENS(S.hcap, sizeof(long long) * (nV + 1));
    ENS(S.hptr, sizeof(long long) * (nV + 1));
    // window rank when the rows' column windows take at most RANK_WORDS_PER_NNZ words per stored
    // entry together, hash tables otherwise (the choice of the first assembly holds in replays)
    ENS(S.rwords, sizeof(long long) * (nV + 1));
    ENS(S.rbase, sizeof(long long) * (nV + 1));
    ENS(S.rlo, sizeof(int) * (nV + 1));
    k_rank_words<<<grid_for(nV, 256), 256, 0, S.st>>>(S.rowptr.get<long long>(), S.cols.get<int>(), nV,
                                                      S.rwords.get<long long>(), S.rlo.get<int>()); ++S.nlaunch;
    int r = scan_excl<long long>(S, S.rwords.get<long long>(), nV, S.rbase.get<long long>());
    if (r) return r;
    r = d2h(S, &S.rtot, S.rbase.get<long long>() + nV, 1);
    if (r) return r;
    if (!S.replay) S.use_rank = S.rtot <= (long long)RANK_WORDS_PER_NNZ * std::max<long long>(nnz, 1);
    if (S.use_rank) {
        ENS(S.rankmap, sizeof(uint2) * (S.rtot + 1));
        k_rank_fill<<<S.nSM * 8, 256, 0, S.st>>>(S.rowptr.get<long long>(), S.cols.get<int>(), nV, S.rbase.get<long long>(),
                                                 S.rlo.get<int>(), S.rankmap.get<uint2>()); ++S.nlaunch;
    } else {
        k_hash_cap<<<grid_for(nV, 256), 256, 0, S.st>>>(S.rowptr.get<long long>(), nV, S.hcap.get<long long>()); ++S.nlaunch;
        r = scan_excl<long long>(S, S.hcap.get<long long>(), nV, S.hptr.get<long long>());
        if (r) return r;
        r = d2h(S, &S.htot, S.hptr.get<long long>() + nV, 1);
        if (r) return r;
        ENS(S.htab, sizeof(unsigned long long) * (S.htot + 1));
        CK(cudaMemsetAsync(S.htab.p, 0xff, sizeof(unsigned long long) * (S.htot + 1), S.st));
        k_hash_fill<<<S.nSM * 8, 256, 0, S.st>>>(S.rowptr.get<long long>(), S.cols.get<int>(), nV, S.hptr.get<long long>(), S.htab.get<unsigned long long>()); ++S.nlaunch;
    }
    if (S.pmode != PM_RETRI) {   // the barycenter pass writes its own rows only: no mirror slots
        CK(cudaGetLastError());
        return NLFEM_OK;
    }
    ENS(S.tpos, sizeof(int) * (nnz + 1));
    if (nnz >= 0x7fffffffLL)
        return fail(NLFEM_ERR_UNSUPPORTED, "the one-sided pass indexes matrix slots with 32-bit integers (2^31 - 1 slots at most)");
    ENS(S.dslot, sizeof(int) * (nE * dV * dV + 1));
    const SlotMap m = slot_map(S);
    k_tpos<<<S.nSM * 8, 256, 0, S.st>>>(m, S.cols.get<int>(), S.labV.get<int>(), nV, S.tpos.get<int>(), S.err.get<int>()); ++S.nlaunch;
    k_dslot<DIM><<<grid_for(nE, 256), 256, 0, S.st>>>(m, S.T32.get<int>(), S.labV.get<int>(), nE, S.dslot.get<int>()); ++S.nlaunch;
    CK(cudaGetLastError());
    return NLFEM_OK;
}

// Rows written in one bitmap pass into a scratch at an atomic cursor (pass 2), its capacity the
// previous assembly's total; with no capacity yet, or after an overflow, the rows are counted
// first (pass 0). Counters[cursor] and err[ovf] are the pass's cursor and overflow flag.
template <int DIM>
static int run_rows_direct(Session &S, RowArgs o, long long nrows, DevBuf &cnt, DevBuf &off, DevBuf &ptr,
                           DevBuf &scratch, long long &cap, int cursor_i, int ovf_i, int words, int threads,
                           unsigned grid, size_t smem) {
    ENS(cnt, sizeof(int) * (nrows + 1));
    ENS(off, sizeof(long long) * (nrows + 1));
    ENS(ptr, sizeof(long long) * (nrows + 1));
    o.rowptr = nullptr; o.cols = nullptr;
    o.rowcnt = cnt.get<int>();
    o.rowoff = off.get<long long>();
    unsigned long long *cursor = S.counters.get<unsigned long long>() + cursor_i;
    int *ovf = S.err.get<int>() + ovf_i;
    int r;
    for (int attempt = 0; attempt < 2; attempt++) {
        if (cap == 0) {   // count the rows first
            o.scratch = nullptr; o.cap = 0; o.cursor = nullptr; o.ovf = nullptr;
            k_row_pattern_bm<DIM><<<grid, threads, smem, S.st>>>(o, 0, words); ++S.nlaunch;
            if ((r = scan_excl<int>(S, cnt.get<int>(), nrows, ptr.get<long long>()))) return r;
            long long tot = 0;
            if ((r = d2h(S, &tot, ptr.get<long long>() + nrows, 1))) return r;
            cap = tot + 1;
        }
        ENS(scratch, sizeof(int) * (cap + 1));
        CK(cudaMemsetAsync(cursor, 0, sizeof(unsigned long long), S.st));
        CK(cudaMemsetAsync(ovf, 0, sizeof(int), S.st));
        o.scratch = scratch.get<int>(); o.cap = cap; o.cursor = cursor; o.ovf = ovf;
        k_row_pattern_bm<DIM><<<grid, threads, smem, S.st>>>(o, 2, words); ++S.nlaunch;
        int of = 0;
        if ((r = d2h(S, &of, ovf, 1))) return r;
        if (!of) return NLFEM_OK;
        if (attempt == 1) return fail(NLFEM_ERR_CUDA, "internal: row scratch overflow after a recount");
        cap = 0;
    }
    return NLFEM_OK;
}

// Per element, the vertices of its partners and its own (none without a partner): the bitmap
// kernel in mode 0 over elements, each element the only member of its own row. The one-sided
// passes' row patterns are then unions of these lists (mode 2).
template <int DIM>
static int run_elem_vlists(Session &S, const RowArgs &a, int words, int threads, unsigned grid, size_t smem) {
    const long long nE = S.nE;
    ENS(S.eid_ptr, sizeof(long long) * (nE + 1));
    ENS(S.eid, sizeof(int) * (nE + 1));
    k_iota_rows<<<grid_for(nE + 1, 256), 256, 0, S.st>>>(nE, S.eid_ptr.get<long long>(), S.eid.get<int>()); ++S.nlaunch;
    RowArgs o = a;
    o.in_ptr = nullptr;
    o.all_rows = 1;
    o.mode = 0;
    o.vptr = S.eid_ptr.get<long long>(); o.vel = S.eid.get<int>(); o.vprob = S.eprob.get<int>(); o.nV = nE;
    int r = run_rows_direct<DIM>(S, o, nE, S.vp_cnt, S.vp_off, S.vp_ptr, S.vp_scratch, S.vp_cap, 15, 11,
                                 words, threads, grid, smem);
    if (r) return r;
    return NLFEM_OK;
}

// Rows of the one-sided retriangulate pass without element in-lists. Row t holds the vertices of
// the partners of t's elements (out-pairs) and of the elements whose partners contain t
// (in-pairs): the second set is {u : t in out-row(u)}, the transpose of the out-pair rows. So
// the out-pair rows of every vertex go to a scratch (one bitmap pass; a first assembly counts
// first), are transposed (count, scan, fill), and the row pass below takes the union of each
// row and its transpose. A scratch overflow (err[10]) recounts.
template <int DIM>
static int run_pattern_transposed(Session &S, RowArgs &a, int words, int threads, unsigned grid, size_t smem) {
    const long long nV = S.nV;
    ENS(S.po_cnt, sizeof(int) * (nV + 1));
    ENS(S.po_off, sizeof(long long) * (nV + 1));
    ENS(S.po_ptr, sizeof(long long) * (nV + 1));
    RowArgs o = a;
    o.in_ptr = nullptr;
    o.all_rows = 1;
    o.mode = S.vlists ? 2 : 0;
    int r = run_rows_direct<DIM>(S, o, nV, S.po_cnt, S.po_off, S.po_ptr, S.po_scratch, S.po_cap, 14, 10,
                                 words, threads, grid, smem);
    if (r) return r;
    ENS(S.tcnt, sizeof(int) * (nV + 1));
    ENS(S.tptr, sizeof(long long) * (nV + 1));
    CK(cudaMemsetAsync(S.tcnt.p, 0, sizeof(int) * (nV + 1), S.st));
    k_tcount<<<S.nSM * 8, 256, 0, S.st>>>(S.po_off.get<long long>(), S.po_cnt.get<int>(), S.po_scratch.get<int>(),
                                          S.labV.get<int>(), nV, S.tcnt.get<int>()); ++S.nlaunch;
    if ((r = scan_excl<int>(S, S.tcnt.get<int>(), nV, S.tptr.get<long long>()))) return r;
    if ((r = d2h(S, &S.t_nnz, S.tptr.get<long long>() + nV, 1))) return r;
    ENS(S.tcols, sizeof(int) * (S.t_nnz + 1));
    CK(cudaMemsetAsync(S.tcnt.p, 0, sizeof(int) * (nV + 1), S.st));
    k_tfill<<<S.nSM * 8, 256, 0, S.st>>>(S.po_off.get<long long>(), S.po_cnt.get<int>(), S.po_scratch.get<int>(),
                                         S.labV.get<int>(), nV, S.tptr.get<long long>(), S.tcnt.get<int>(),
                                         S.tcols.get<int>()); ++S.nlaunch;
    CK(cudaGetLastError());
    a.mode = 1;
    a.all_rows = 0;
    a.srcoff = S.po_off.get<long long>(); a.srccnt = S.po_cnt.get<int>(); a.srccols = S.po_scratch.get<int>();
    a.tptr = S.tptr.get<long long>(); a.tcols = S.tcols.get<int>();
    return NLFEM_OK;
}

template <int DIM>
static int run_pattern_bm(Session &S, int words, int threads) {
    const long long nV = S.nV;
    ENS(S.rowcnt, sizeof(int) * (nV + 1));
    ENS(S.rowptr, sizeof(long long) * (nV + 1));
    RowArgs a;
    memset(&a, 0, sizeof(a));
    a.T32 = S.T32.get<int>(); a.labT = S.labT.get<int>(); a.labV = S.labV.get<int>();
    a.vprob = S.vprob.get<int>(); a.vel = S.vel.get<int>(); a.pB = S.pB.get<int>(); a.inA = S.inA.get<int>();
    a.vptr = S.vptr.get<long long>(); a.out_ptr = S.out_ptr.get<long long>();
    if (S.pairs_pool) { a.pB = S.pool.get<int>(); a.out_ptr = S.seg_start.get<long long>(); a.out_cnt = S.seg_cnt.get<int>(); }
    a.in_ptr = S.pmode == PM_BARY ? nullptr : S.in_ptr.get<long long>();   // rows of one-sided rules: out-pairs only
    a.probs = S.prm.get<ProbParams>(); a.nV = nV;
    a.marks = nullptr; a.mstride = 0;
    a.rowptr = nullptr; a.cols = nullptr; a.rowcnt = S.rowcnt.get<int>();
    a.scratch = nullptr; a.cap = 0; a.cursor = nullptr; a.rowoff = nullptr; a.ovf = nullptr;
    const size_t smem = (size_t)words * 4 * (threads / 32);
    CK(cudaFuncSetAttribute(k_row_pattern_bm<DIM>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int per_sm = 0;
    CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_row_pattern_bm<DIM>, threads, smem));
    const unsigned grid = (unsigned)(S.nSM * std::max(per_sm, 1));
    if (S.hint_nE == S.nE && S.hint_nV == S.nV) {   // one-shot calls: the previous call's sizes
        if (S.pat_cap == 0) S.pat_cap = S.hint_pat_cap;
        if (S.po_cap == 0) S.po_cap = S.hint_po_cap;
        if (S.vp_cap == 0) S.vp_cap = S.hint_vp_cap;
    }
    // the one-sided passes' rows (out-pairs only) are unions of per-element vertex lists
    S.vlists = S.pmode == PM_RETRI || S.pmode == PM_BARY;
    if (S.vlists) {
        int r = run_elem_vlists<DIM>(S, a, words, threads, grid, smem);
        if (r) return r;
        a.vpool = S.vp_scratch.get<int>(); a.vseg_start = S.vp_off.get<long long>(); a.vseg_cnt = S.vp_cnt.get<int>();
        if (S.pmode == PM_BARY) a.mode = 2;
    }
    if (S.pmode == PM_RETRI) {
        int r = run_pattern_transposed<DIM>(S, a, words, threads, grid, smem);
        if (r) return r;
    }
    if (S.pat_cap > 0) {
        // single bitmap pass: rows go to a scratch of the previous assembly's size, then a copy
        // puts them in CSR order; a scratch overflow falls back to the two passes below
        ENS(S.rowoff, sizeof(long long) * (nV + 1));
        ENS(S.pscratch, sizeof(int) * (S.pat_cap + 1));
        unsigned long long *cursor = S.counters.get<unsigned long long>() + 11;
        CK(cudaMemsetAsync(cursor, 0, sizeof(unsigned long long), S.st));
        CK(cudaMemsetAsync(S.err.get<int>() + 6, 0, sizeof(int), S.st));
        a.scratch = S.pscratch.get<int>(); a.cap = S.pat_cap; a.cursor = cursor;
        a.rowoff = S.rowoff.get<long long>(); a.ovf = S.err.get<int>() + 6;
        k_row_pattern_bm<DIM><<<grid, threads, smem, S.st>>>(a, 2, words); ++S.nlaunch;
        int r = scan_excl<int>(S, S.rowcnt.get<int>(), nV, S.rowptr.get<long long>());
        if (r) return r;
        int ovf = 0;
        if ((r = d2h(S, &ovf, S.err.get<int>() + 6, 1))) return r;
        if (!ovf) {
            if ((r = d2h(S, &S.nnz_struct, S.rowptr.get<long long>() + nV, 1))) return r;
            ENS(S.cols, sizeof(int) * (S.nnz_struct + 1));
            k_row_copy<<<S.nSM * 8, 256, 0, S.st>>>(S.rowptr.get<long long>(), S.rowoff.get<long long>(), nV,
                                                    S.pscratch.get<int>(), S.cols.get<int>()); ++S.nlaunch;
            CK(cudaGetLastError());
            S.stats.nnz_structural = (long)S.nnz_struct;
            if (S.pmode == PM_RETRI || S.pmode == PM_BARY) return run_slot_maps<DIM>(S);
            return NLFEM_OK;
        }
        a.scratch = nullptr; a.cap = 0; a.cursor = nullptr; a.rowoff = nullptr; a.ovf = nullptr;
    }
    k_row_pattern_bm<DIM><<<grid, threads, smem, S.st>>>(a, 0, words); ++S.nlaunch;
    int r = scan_excl<int>(S, S.rowcnt.get<int>(), nV, S.rowptr.get<long long>());
    if (r) return r;
    r = d2h(S, &S.nnz_struct, S.rowptr.get<long long>() + nV, 1);
    if (r) return r;
    ENS(S.cols, sizeof(int) * (S.nnz_struct + 1));
    a.rowptr = S.rowptr.get<long long>(); a.cols = S.cols.get<int>();
    k_row_pattern_bm<DIM><<<grid, threads, smem, S.st>>>(a, 1, words); ++S.nlaunch;
    CK(cudaGetLastError());
    S.stats.nnz_structural = (long)S.nnz_struct;
    S.pat_cap = S.nnz_struct;   // the next assembly builds the pattern in one pass
    ENS(S.rowoff, sizeof(long long) * (nV + 1));
    ENS(S.pscratch, sizeof(int) * (S.pat_cap + 1));
    if (S.pmode == PM_RETRI || S.pmode == PM_BARY) return run_slot_maps<DIM>(S);
    return NLFEM_OK;
}

template <int DIM>
static int run_pattern(Session &S) {
    const long long nV = S.nV;
    // bitmap marks in shared memory when a problem's vertex bitmap is small enough
    const int words = (S.maxNV + 31) / 32;
    const int bm_threads = pattern_bitmap_threads(S);
    if (bm_threads) return run_pattern_bm<DIM>(S, words, bm_threads);
    const int nwarps = S.nSM * 4 * 8;
    ENS(S.marks, sizeof(unsigned) * (size_t)nwarps * S.maxNV);
    ENS(S.rowcnt, sizeof(int) * (nV + 1));
    ENS(S.rowptr, sizeof(long long) * (nV + 1));
    CK(cudaMemsetAsync(S.marks.p, 0, sizeof(unsigned) * (size_t)nwarps * S.maxNV, S.st));
    RowArgs a;
    a.T32 = S.T32.get<int>(); a.labT = S.labT.get<int>(); a.labV = S.labV.get<int>();
    a.vprob = S.vprob.get<int>(); a.vel = S.vel.get<int>(); a.pB = S.pB.get<int>(); a.inA = S.inA.get<int>();
    a.vptr = S.vptr.get<long long>(); a.out_ptr = S.out_ptr.get<long long>();
    a.in_ptr = S.pmode == PM_BARY ? nullptr : S.in_ptr.get<long long>();   // rows of one-sided rules: out-pairs only
    a.probs = S.prm.get<ProbParams>(); a.nV = nV;
    a.marks = S.marks.get<unsigned>(); a.mstride = S.maxNV;
    a.rowptr = nullptr; a.cols = nullptr; a.rowcnt = S.rowcnt.get<int>();
    k_row_pattern<DIM><<<S.nSM * 4, 256, 0, S.st>>>(a, 0); ++S.nlaunch;
    int r = scan_excl<int>(S, S.rowcnt.get<int>(), nV, S.rowptr.get<long long>());
    if (r) return r;
    r = d2h(S, &S.nnz_struct, S.rowptr.get<long long>() + nV, 1);
    if (r) return r;
    ENS(S.cols, sizeof(int) * (S.nnz_struct + 1));
    a.rowptr = S.rowptr.get<long long>(); a.cols = S.cols.get<int>();
    k_row_pattern<DIM><<<S.nSM * 4, 256, 0, S.st>>>(a, 1); ++S.nlaunch;
    const int cap = 16384;
    CK(cudaFuncSetAttribute(k_row_sort, cudaFuncAttributeMaxDynamicSharedMemorySize, cap * (int)sizeof(int)));
    k_row_sort<<<S.nSM * 4, 256, cap * sizeof(int), S.st>>>(S.rowptr.get<long long>(), nV, S.cols.get<int>(), cap); ++S.nlaunch;
    k_row_sort_global<<<S.nSM * 4, 256, 0, S.st>>>(S.rowptr.get<long long>(), nV, S.cols.get<int>(), cap); ++S.nlaunch;
    CK(cudaGetLastError());
    S.stats.nnz_structural = (long)S.nnz_struct;
    if (S.pmode == PM_RETRI || S.pmode == PM_BARY) return run_slot_maps<DIM>(S);
    return NLFEM_OK;
}

static int check_errors(Session &S);

static Duffy duffy_view(const Session &S) {
    Duffy d;
    const int nPg = S.duffy_nPg;
    const int nTr[3] = {2, 5, 6};
    const double *h = S.duffy.get<double>();
    size_t o = 0;
    for (int c = 0; c < 3; c++) {
        d.alpha[c] = h + o; o += (size_t)nTr[c] * nPg * 4;
        d.tdet[c] = h + o; o += (size_t)nTr[c] * nPg;
        d.alphaU[c] = h + o; o += (size_t)nTr[c] * nPg * 4;
        d.tdetW[c] = h + o; o += (size_t)nTr[c] * nPg;
    }
    d.dg = h + o;
    d.nPg = nPg;
    const float *f = S.duffyf.get<float>();
    size_t of = 0;
    for (int c = 0; c < 3; c++) {
        d.alf[c] = reinterpret_cast<const float4 *>(f + of); of += (size_t)nTr[c] * nPg * 4;
        d.wf[c] = f + of; of += ((size_t)nTr[c] * nPg + 3) / 4 * 4;
        d.alfU[c] = reinterpret_cast<const float4 *>(f + of); of += (size_t)nTr[c] * nPg * 4;
        d.wfW[c] = f + of; of += ((size_t)nTr[c] * nPg + 3) / 4 * 4;
    }
    return d;
}

__global__ void k_iota(int *l, long long n) {
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) l[i] = (int)i;
}

// Blocks of explicit pairs (no scatter): the kernel-level parity hook.
template <int DIM>
static int run_pair_blocks(Session &S, long long n, const long *pairs, int close, double *out, int *ret) {
    constexpr int dV = DIM + 1;
    int r = run_prep<DIM>(S);
    if (r) return r;
    std::vector<int> a32(n), b32(n);
    for (long long i = 0; i < n; i++) {
        if (pairs[2 * i] < 0 || pairs[2 * i] >= S.nE || pairs[2 * i + 1] < 0 || pairs[2 * i + 1] >= S.nE)
            return fail(NLFEM_ERR_INVALID, "pair index out of range");
        a32[i] = (int)pairs[2 * i];
        b32[i] = (int)pairs[2 * i + 1];
    }
    ENS(S.pA, sizeof(int) * (n + 1));
    ENS(S.pB, sizeof(int) * (n + 1));
    ENS(S.vals, sizeof(double) * 4 * dV * dV * (n + 1));
    ENS(S.keepcnt, sizeof(int) * (n + 1));
    ENS(S.closelist, sizeof(int) * (n + 1));
    CK(cudaMemcpyAsync(S.pA.p, a32.data(), sizeof(int) * n, cudaMemcpyHostToDevice, S.st));
    CK(cudaMemcpyAsync(S.pB.p, b32.data(), sizeof(int) * n, cudaMemcpyHostToDevice, S.st));
    CK(cudaMemsetAsync(S.vals.p, 0, sizeof(double) * 4 * dV * dV * (n + 1), S.st));
    QuadArgs a;
    memset(&a, 0, sizeof(a));
    a.pA = S.pA.get<int>(); a.pB = S.pB.get<int>(); a.T32 = S.T32.get<int>(); a.labV = S.labV.get<int>();
    a.labT = S.labT.get<int>();
    a.eprob = S.eprob.get<int>(); a.EC = S.EC.get<double>(); a.adet = S.adet.get<double>();
    a.probs = S.prm.get<ProbParams>(); a.P = n; a.err = S.err.get<int>();
    a.n_close = S.counters.get<unsigned long long>() + 4;
    a.blocks_out = S.vals.get<double>(); a.ret_out = S.keepcnt.get<int>(); a.force_close = close;
    const ProbParams &P0 = S.hprm[0];
    const int method = close ? P0.close : P0.remote;
    if (method == MTH_FRACTIONAL || method == MTH_WEAKSING) {
        if (DIM != 2 || S.duffy_nPg == 0) return fail(NLFEM_ERR_INVALID, "close rule needs a 2D mesh and a tensor Gauss rule");
        k_iota<<<grid_for(n, 256), 256, 0, S.st>>>(S.closelist.get<int>(), n); ++S.nlaunch;
        a.list = S.closelist.get<int>();
        a.nlist = n;
        k_quad_close<false><<<grid_for(n * 32, 128), 128, 0, S.st>>>(a, duffy_view(S)); ++S.nlaunch;
    } else {
        k_quad_fp64<DIM><<<grid_for(n, 128), 128, 0, S.st>>>(a, S.rule); ++S.nlaunch;
    }
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(S.st));
    r = check_errors(S);
    if (r) return r;
    r = d2h(S, out, S.vals.get<double>(), (size_t)n * 4 * dV * dV);
    if (r) return r;
    return d2h(S, ret, S.keepcnt.get<int>(), (size_t)n);
}

template <typename R>
static PassRuleT<R> make_pass_rule(const Rule &r, int dim) {
    PassRuleT<R> pr;
    memset(&pr, 0, sizeof(pr));
    const int dV = dim + 1, NS = dV * (dV + 1) / 2;
    for (int k = 0; k < r.nPx; k++) {
        pr.dxf[k] = (R)r.dx[k];
        int t = 0;
        for (int a = 0; a < dV; a++) {
            pr.cx[dV * k + a] = (R)(r.dx[k] * r.psix[dV * k + a]);
            for (int b = a; b < dV; b++) pr.cxx[NS * k + t++] = (R)(r.dx[k] * r.psix[dV * k + a] * r.psix[dV * k + b]);
        }
    }
    double insum[1 + 4 + 10] = {0}, mom[6] = {0};
    for (int i = 0; i < r.nPy; i++) {
        for (int c = 0; c < dim; c++) pr.pyf[dim * i + c] = (R)r.Py[dim * i + c];
        int t = 0;
        insum[0] += r.dy[i];
        for (int a = 0; a < dV; a++) {
            pr.cy[dV * i + a] = (R)(r.dy[i] * r.psiy[dV * i + a]);
            insum[1 + a] += r.dy[i] * r.psiy[dV * i + a];
            for (int b = a; b < dV; b++) {
                insum[1 + dV + t] += r.dy[i] * r.psiy[dV * i + a] * r.psiy[dV * i + b];
                pr.cyy[NS * i + t++] = (R)(r.dy[i] * r.psiy[dV * i + a] * r.psiy[dV * i + b]);
            }
        }
        if (dim == 2) {
            const double px = r.Py[2 * i], py = r.Py[2 * i + 1], w = r.dy[i];
            mom[0] += w; mom[1] += w * px; mom[2] += w * py;
            mom[3] += w * px * px; mom[4] += w * px * py; mom[5] += w * py * py;
        }
    }
    for (int q = 0; q < 1 + 4 + 10; q++) pr.insum[q] = (R)insum[q];
    for (int q = 0; q < 6; q++) pr.mom[q] = (R)mom[q];
    double xsum[10 + 4 + 1] = {0};
    for (int k = 0; k < r.nPx; k++) {
        int t = 0;
        for (int a = 0; a < dV; a++) {
            xsum[NS + a] += r.dx[k] * r.psix[dV * k + a];
            for (int b = a; b < dV; b++) xsum[t++] += r.dx[k] * r.psix[dV * k + a] * r.psix[dV * k + b];
        }
        xsum[NS + dV] += r.dx[k];
    }
    for (int q = 0; q < NS + dV + 1; q++) pr.xsum[q] = (R)xsum[q];
    return pr;
}

// Close pairs of the singular kernel: Duffy blocks into closebuf (FP64, one warp per pair).
static int run_close(Session &S) {
    if (S.dim != 2 || S.duffy_nPg == 0) return NLFEM_OK;
    const long long nE = S.nE;
    const long long nslot = S.nadj + nE;
    ENS(S.closeA, sizeof(int) * (nslot + 1));
    ENS(S.closeB, sizeof(int) * (nslot + 1));
    ENS(S.closebuf, sizeof(double) * 36 * (nslot + 1));
    ENS(S.closelist, sizeof(int) * (nslot + 1));
    k_close_pairs<<<grid_for(nE, 256), 256, 0, S.st>>>(S.xadj.get<long long>(), S.adj.get<int>(), S.labT.get<int>(), S.eprob.get<int>(), S.prm.get<ProbParams>(), nE, S.closeA.get<int>(), S.closeB.get<int>()); ++S.nlaunch;
    QuadArgs a;
    memset(&a, 0, sizeof(a));
    // under DG the rows are element DOFs (S.T32) and the close pairs are found on the vertices
    a.pA = S.closeA.get<int>(); a.pB = S.closeB.get<int>(); a.T32 = S.dg_rows ? S.dgT32.get<int>() : S.T32.get<int>();
    a.labV = S.labV.get<int>();
    a.labT = S.labT.get<int>();
    a.eprob = S.eprob.get<int>(); a.EC = S.EC.get<double>(); a.adet = S.adet.get<double>();
    a.probs = S.prm.get<ProbParams>(); a.P = nslot; a.err = S.err.get<int>();
    a.n_close = S.counters.get<unsigned long long>() + 4;
    a.blocks_out = S.closebuf.get<double>(); a.ret_out = S.closelist.get<int>(); a.force_close = 1;
    k_iota<<<grid_for(nslot, 256), 256, 0, S.st>>>(S.closelist.get<int>(), nslot); ++S.nlaunch;
    a.list = S.closelist.get<int>();
    a.nlist = nslot;
    // the mixed path takes the kernel power in FP32 after an exact binary range reduction
    if (S.prec == PREC_MIX) k_quad_close<true><<<grid_for(nslot * 32, 128), 128, 0, S.st>>>(a, duffy_view(S));
    else k_quad_close<false><<<grid_for(nslot * 32, 128), 128, 0, S.st>>>(a, duffy_view(S));
    ++S.nlaunch;
    CK(cudaGetLastError());
    return NLFEM_OK;
}

// One-sided mixed passes (passes_mix.cuh, passes_bary.cuh): one persistent launch over all
// elements. kconst is the closed-form instance for constant kernels, kgen the general one. A batch
// that mixes kernels runs both, each over its problems' elements (constant-kernel elements listed
// first), so every problem goes through the same code as its single assembly and the batch matrices
// equal the single ones bit for bit. A contribution outside the fixed-point range sets err[5]; the
// pass is then redone with a unit 2^16 times coarser.
template <typename PR>
using OneSidedKernelT = void (*)(MixArgs, Rule, PR);
typedef OneSidedKernelT<PassRule> OneSidedKernel;
// Kernel class of a problem for the one-sided passes: 0 constant kernel (closed forms), 1 other
// regular kernel, 2 singular kernel with Duffy close pairs.
static int kernel_class(const ProbParams &q) {
    if (q.kernel == KER_CONSTANT || q.kernel == KER_CONSTANT3D) return 0;
    return duffy_close(q) ? 2 : 1;
}

template <typename PR>
static int run_pass_one_sided(Session &S, const PassArgs &pa, const PR &pr, const OneSidedKernelT<PR> *kfn,
                              int threads, size_t smem) {
    const long long nnz = S.nnz_struct;
    int ncls[3] = {0, 0, 0};
    for (const ProbParams &q : S.hprm) ncls[kernel_class(q)]++;
    struct Launch { OneSidedKernelT<PR> k; const int *list; int count; int per_sm; };
    Launch L[3];
    int nl = 0;
    for (int c = 0; c < 3; c++)
        if (ncls[c] == (int)S.hprm.size()) L[nl++] = Launch{kfn[c], nullptr, (int)S.nE, 0};
    if (nl == 0) {   // several classes: one launch per class over its problems' elements
        if (S.kc_off[0] < 0) {
            if (S.replay) return fail(NLFEM_ERR_UNSUPPORTED, "element list by kernel class missing in graph capture");
            std::vector<int> h;
            h.reserve((size_t)S.nE);
            for (int c = 0; c < 3; c++) {
                S.kc_off[c] = (long long)h.size();
                for (const ProbParams &q : S.hprm)
                    if (kernel_class(q) == c)
                        for (int e = 0; e < q.nE; e++) h.push_back(q.elem_off + e);
            }
            S.kc_off[3] = (long long)h.size();
            ENS(S.kclist, sizeof(int) * (h.size() + 1));
            CK(cudaMemcpyAsync(S.kclist.p, h.data(), sizeof(int) * h.size(), cudaMemcpyHostToDevice, S.st));
            CK(cudaStreamSynchronize(S.st));
        }
        const int *lst = S.kclist.get<int>();
        for (int c = 0; c < 3; c++)
            if (S.kc_off[c + 1] > S.kc_off[c])
                L[nl++] = Launch{kfn[c], lst + S.kc_off[c], (int)(S.kc_off[c + 1] - S.kc_off[c]), 0};
    }
    for (int i = 0; i < nl; i++) {
        CK(cudaFuncSetAttribute(L[i].k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&L[i].per_sm, L[i].k, threads, smem));
        if (L[i].per_sm < 1) return fail(NLFEM_ERR_UNSUPPORTED, "quadrature rule too large for the pass's shared memory");
        if (S.tune_pass > 0) L[i].per_sm = std::min(L[i].per_sm, S.tune_pass);   // autotuned
        S.used_pass = std::max(i ? S.used_pass : 0, L[i].per_sm);
    }
    MixArgs ma;
    ma.p = pa;
    ma.m = slot_map(S);
    ma.work = reinterpret_cast<int *>(S.counters.get<unsigned long long>() + 10);
    ma.valsN = nullptr;
    ma.elp = nullptr;
    const bool retri = S.pmode == PM_RETRI;
    if (retri) {
        ENS(S.valsN, sizeof(long long) * (nnz + 1));
        ENS(S.elp, sizeof(long long) * 6 * (S.nE + 1));
        ma.valsN = S.valsN.get<long long>();
        ma.elp = S.elp.get<long long>();
    }
    for (int attempt = 0; attempt < 4; attempt++) {
        CK(cudaMemsetAsync(S.vals.p, 0, sizeof(long long) * (nnz + 1), S.st));
        if (retri) {
            CK(cudaMemsetAsync(S.valsN.p, 0, sizeof(long long) * (nnz + 1), S.st));
            CK(cudaMemsetAsync(S.elp.p, 0, sizeof(long long) * 6 * (S.nE + 1), S.st));
        }
        CK(cudaMemsetAsync(S.err.get<int>() + 5, 0, sizeof(int), S.st));
        CK(cudaMemsetAsync(S.counters.get<unsigned long long>() + 4, 0, 3 * sizeof(unsigned long long), S.st));
        CK(cudaMemsetAsync(S.counters.get<unsigned long long>() + 12, 0, 2 * sizeof(unsigned long long), S.st));
        for (int i = 0; i < nl; i++) {
            if (L[i].count == 0) continue;
            ma.p.list = L[i].list;
            ma.p.count = L[i].count;
            CK(cudaMemsetAsync(ma.work, 0, sizeof(int), S.st));
            L[i].k<<<(unsigned)(S.nSM * L[i].per_sm), threads, smem, S.st>>>(ma, S.rule, pr); ++S.nlaunch;
            CK(cudaGetLastError());
        }
        if (retri) {   // termLocalPrime blocks, then the transposed termNonloc sums
            long long *vals = reinterpret_cast<long long *>(S.vals.p);
            k_elem_blocks<<<grid_for(S.nE, 256), 256, 0, S.st>>>(ma.elp, S.dslot.get<int>(), S.T32.get<int>(), S.labV.get<int>(), S.nE, vals, S.err.get<int>()); ++S.nlaunch;
            k_sym_add<<<S.nSM * 16, 256, 0, S.st>>>(S.rowptr.get<long long>(), S.cols.get<int>(), S.tpos.get<int>(), ma.valsN, S.nV, vals); ++S.nlaunch;
            CK(cudaGetLastError());
        }
        if (S.pmode == PM_BARY) {   // the diagonal entries from the row sums
            k_row_diag<<<S.nSM * 16, 256, 0, S.st>>>(S.rowptr.get<long long>(), S.cols.get<int>(), S.nV,
                                                     reinterpret_cast<long long *>(S.vals.p)); ++S.nlaunch;
            CK(cudaGetLastError());
        }
        if (S.replay) return NLFEM_OK;   // the overflow flag is checked after the replay
        int ovf = 0;
        int r = d2h(S, &ovf, S.err.get<int>() + 5, 1);
        if (r) return r;
        if (!ovf) return NLFEM_OK;
        for (ProbParams &q : S.hprm) {
            r = set_fx_unit(q, q.fx_ue - (q.scale_exp + FX_GUARD - 62) + 16);
            if (r) return r;
        }
        CK(cudaMemcpyAsync(S.prm.p, S.hprm.data(), sizeof(ProbParams) * S.hprm.size(), cudaMemcpyHostToDevice, S.st));
    }
    return fail(NLFEM_ERR_NUMERIC, "contribution outside the fixed-point range (non-finite value?)");
}

// Vector-valued kernels: one thread per ordered pair, FP64 blocks, 128-bit fixed-point sums in the
// expanded slots (od^2 per structural entry).
template <int DIM>
static int run_pass_vec(Session &S) {
    const long long nslot = (long long)S.od * S.od * S.nnz_struct;
    ENS(S.vacc, sizeof(unsigned long long) * 2 * (nslot + 1));
    ENS(S.vtiny, sizeof(unsigned) * (nslot + 1));
    CK(cudaMemsetAsync(S.vacc.p, 0, sizeof(unsigned long long) * 2 * (nslot + 1), S.st));
    CK(cudaMemsetAsync(S.vtiny.p, 0, sizeof(unsigned) * (nslot + 1), S.st));
    unsigned long long *cnt = S.counters.get<unsigned long long>();
    VecArgs a;
    memset(&a, 0, sizeof(a));
    a.pA = S.pA.get<int>(); a.pB = S.pB.get<int>(); a.T32 = S.T32.get<int>(); a.labV = S.labV.get<int>();
    a.labT = S.labT.get<int>(); a.eprob = S.eprob.get<int>(); a.EC = S.EC.get<double>(); a.adet = S.adet.get<double>();
    a.probs = S.prm.get<ProbParams>(); a.rowptr = S.rowptr.get<long long>(); a.cols = S.cols.get<int>();
    a.acc = S.vacc.get<unsigned long long>(); a.tiny = S.vtiny.get<unsigned>(); a.P = S.P; a.err = S.err.get<int>();
    a.n_close = cnt + 4; a.n_subtri = cnt + 5;
    Duffy d;
    memset(&d, 0, sizeof(d));
    if (S.duffy_nPg) d = duffy_view(S);
    if (S.P > 0) {
        if (DIM == 2 && S.od == 2) k_quad_vec<2, 2><<<grid_for(S.P, 128), 128, 0, S.st>>>(a, S.rule, d);
        else if (DIM == 3 && S.od == 3) k_quad_vec<3, 3><<<grid_for(S.P, 128), 128, 0, S.st>>>(a, S.rule, d);
        else return fail(NLFEM_ERR_UNSUPPORTED, "vector-valued kernels: outdim 2 in 2D or 3 in 3D");
        ++S.nlaunch;
    }
    CK(cudaGetLastError());
    return NLFEM_OK;
}

// Finish of the vector path: expanded rows od v + i, exact zeros dropped.
static int run_finish_vec(Session &S) {
    const long long K = (long long)S.od * S.nV;
    ENS(S.keepcnt, sizeof(int) * (K + 1));
    ENS(S.fptr, sizeof(long long) * (K + 1));
    const unsigned grid = (unsigned)grid_for(K * 32, 256);
    if (S.od == 2)
        k_vec_finish_count<2><<<grid, 256, 0, S.st>>>(S.rowptr.get<long long>(), S.nV, S.labV.get<int>(), S.vacc.get<unsigned long long>(), S.vprob.get<int>(), S.prm.get<ProbParams>(), S.keepcnt.get<int>());
    else
        k_vec_finish_count<3><<<grid, 256, 0, S.st>>>(S.rowptr.get<long long>(), S.nV, S.labV.get<int>(), S.vacc.get<unsigned long long>(), S.vprob.get<int>(), S.prm.get<ProbParams>(), S.keepcnt.get<int>());
    ++S.nlaunch;
    int r = scan_excl<int>(S, S.keepcnt.get<int>(), K, S.fptr.get<long long>());
    if (r) return r;
    r = d2h(S, &S.nnz, S.fptr.get<long long>() + K, 1);
    if (r) return r;
    ENS(S.fcols, sizeof(int) * (S.nnz + 1));
    ENS(S.fvals, sizeof(double) * (S.nnz + 1));
    if (S.od == 2)
        k_vec_finish_compact<2><<<grid, 256, 0, S.st>>>(S.rowptr.get<long long>(), S.nV, S.labV.get<int>(), S.cols.get<int>(), S.vacc.get<unsigned long long>(), S.vprob.get<int>(), S.prm.get<ProbParams>(), S.fptr.get<long long>(), S.fcols.get<int>(), S.fvals.get<double>());
    else
        k_vec_finish_compact<3><<<grid, 256, 0, S.st>>>(S.rowptr.get<long long>(), S.nV, S.labV.get<int>(), S.cols.get<int>(), S.vacc.get<unsigned long long>(), S.vprob.get<int>(), S.prm.get<ProbParams>(), S.fptr.get<long long>(), S.fcols.get<int>(), S.fvals.get<double>());
    ++S.nlaunch;
    CK(cudaGetLastError());
    return NLFEM_OK;
}

template <int DIM>
static int run_passes(Session &S) {
    constexpr int dV = DIM + 1;
    const long long nnz = S.nnz_struct;
    ENS(S.vals, sizeof(double) * (nnz + 1));
    CK(cudaMemsetAsync(S.vals.p, 0, sizeof(double) * (nnz + 1), S.st));
    if (S.prec == PREC_MIX && S.pmode == PM_COLORED) {
        ENS(S.touched, (size_t)nnz + 16);
        CK(cudaMemsetAsync(S.touched.p, 0, (size_t)nnz + 16, S.st));
    }
    unsigned long long *cnt = S.counters.get<unsigned long long>();
    CK(cudaMemsetAsync(cnt + 4, 0, 3 * sizeof(unsigned long long), S.st));
    CK(cudaMemsetAsync(cnt + 12, 0, 2 * sizeof(unsigned long long), S.st));
    int r = run_close(S);
    if (r) return r;
    PassArgs a;
    memset(&a, 0, sizeof(a));
    a.T32 = S.T32.get<int>(); a.labV = S.labV.get<int>(); a.eprob = S.eprob.get<int>(); a.labT = S.labT.get<int>();
    a.Tv = S.dg_rows ? S.dgT32.get<int>() : a.T32;
    a.EC = S.EC.get<double>(); a.adet = S.adet.get<double>(); a.EChi = S.EChi.get<float>(); a.EClo = S.EClo.get<float>(); a.BCf = S.BCf.get<float>();
    a.adetf = S.adetf.get<float>();
    a.probs = S.prm.get<ProbParams>(); a.out_ptr = S.out_ptr.get<long long>(); a.in_ptr = S.in_ptr.get<long long>();
    a.pB = S.pB.get<int>(); a.inA = S.inA.get<int>(); a.rowptr = S.rowptr.get<long long>(); a.cols = S.cols.get<int>();
    if (S.pairs_pool) { a.pB = S.pool.get<int>(); a.out_ptr = S.seg_start.get<long long>(); a.out_cnt = S.seg_cnt.get<int>(); }
    a.vals = S.vals.get<double>(); a.xadj = S.xadj.get<long long>(); a.adj = S.adj.get<int>();
    a.closebuf = S.closebuf.get<double>(); a.err = S.err.get<int>();
    a.zptr = S.zptr.get<long long>(); a.zidx = S.zidx.get<long long>();
    a.n_subtri = cnt + 5; a.n_amb = cnt + 6; a.n_close = cnt + 4; a.n_in = cnt + 12; a.n_cut = cnt + 13;
    a.touched = S.prec == PREC_MIX && S.pmode == PM_COLORED ? S.touched.get<unsigned char>() : nullptr;
    if (S.pmode == PM_VEC) return run_pass_vec<DIM>(S);
    const PassRule pr = make_pass_rule<float>(S.rule, DIM);
    if (S.pmode == PM_RETRI && S.onesided64) {
        const PassRuleT<double> pr64 = make_pass_rule<double>(S.rule, DIM);
        const OneSidedKernelT<PassRuleT<double>> k[3] = {k_pass_mix2d<MIX_CONST, double>, k_pass_mix2d<MIX_REGULAR, double>,
                                                        k_pass_mix2d<MIX_SINGULAR, double>};
        return run_pass_one_sided(S, a, pr64, k, MIX_THREADS, mix_warp_bytes<double>(S.rule.nPx) * MIX_WARPS);
    }
    if (S.pmode == PM_RETRI) {
        const OneSidedKernel k[3] = {k_pass_mix2d<MIX_CONST, float>, k_pass_mix2d<MIX_REGULAR, float>,
                                     k_pass_mix2d<MIX_SINGULAR, float>};
        return run_pass_one_sided(S, a, pr, k, MIX_THREADS, mix_warp_bytes<float>(S.rule.nPx) * MIX_WARPS);
    }
    if (S.pmode == PM_BARY) {   // no singular kernels here
        const OneSidedKernel k[3] = {k_pass_bary<DIM, true>, k_pass_bary<DIM, false>, k_pass_bary<DIM, false>};
        return run_pass_one_sided(S, a, pr, k, BARY_THREADS, bary_warp_bytes<DIM>(S.rule.nPx) * BARY_WARPS);
    }
    const size_t smem = sizeof(int) * PASS_WARPS * dV * ROWCACHE;
    if (S.prec == PREC_MIX) CK(cudaFuncSetAttribute(k_pass<DIM, PREC_MIX>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    else CK(cudaFuncSetAttribute(k_pass<DIM, PREC_F64>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    const int ncol = (int)S.color_off.size() - 1;
    for (int c = 0; c < ncol; c++) {
        a.list = S.colorlist.get<int>() + S.color_off[c];
        a.count = S.color_off[c + 1] - S.color_off[c];
        if (!a.count) continue;
        const unsigned grid = (unsigned)std::min<long long>((a.count + PASS_WARPS - 1) / PASS_WARPS, (long long)S.nSM * 8);
        if (S.prec == PREC_MIX) k_pass<DIM, PREC_MIX><<<grid, PASS_THREADS, smem, S.st>>>(a, S.rule, pr);
        else k_pass<DIM, PREC_F64><<<grid, PASS_THREADS, smem, S.st>>>(a, S.rule, pr);
        ++S.nlaunch;
    }
    CK(cudaGetLastError());
    return NLFEM_OK;
}

static int run_finish(Session &S) {
    if (S.pmode == PM_VEC) return run_finish_vec(S);
    const long long nV = S.nV;
    ENS(S.keepcnt, sizeof(int) * (nV + 1));
    ENS(S.fptr, sizeof(long long) * (nV + 1));
    // values: FP64 sums, double-float sums with touched flags (two-sided mixed passes), or
    // fixed-point sums of the one-sided pass (every structural slot received a contribution)
    const int vmode = S.pmode != PM_COLORED ? VAL_FX : (S.prec == PREC_MIX ? VAL_DF : VAL_F64);
    const unsigned char *tch = vmode == VAL_DF ? S.touched.get<unsigned char>() : nullptr;
    const FinishArgs fa{vmode, tch, S.vprob.get<int>(), S.prm.get<ProbParams>()};
    k_finish_count<<<grid_for(nV * 32, 256), 256, 0, S.st>>>(S.rowptr.get<long long>(), nV, S.vals.get<double>(), fa, S.keepcnt.get<int>()); ++S.nlaunch;
    int r = scan_excl<int>(S, S.keepcnt.get<int>(), nV, S.fptr.get<long long>());
    if (r) return r;
    r = d2h(S, &S.nnz, S.fptr.get<long long>() + nV, 1);
    if (r) return r;
    ENS(S.fcols, sizeof(int) * (S.nnz + 1));
    ENS(S.fvals, sizeof(double) * (S.nnz + 1));
    k_finish_compact<<<grid_for(nV * 32, 256), 256, 0, S.st>>>(S.rowptr.get<long long>(), nV, S.cols.get<int>(), S.vals.get<double>(), fa, S.fptr.get<long long>(), S.fcols.get<int>(), S.fvals.get<double>()); ++S.nlaunch;
    CK(cudaGetLastError());
    return NLFEM_OK;
}

static int check_errors(Session &S) {
    int he[8];
    int r = d2h(S, he, S.err.get<int>(), 8);
    if (r) return r;
    if (he[3]) return fail(NLFEM_ERR_CUDA, "internal: CSR slot not found during scatter");
    if (he[4]) return fail(NLFEM_ERR_NUMERIC, "in solve2x2. Matrix not invertible.");
    if (he[7]) return fail(NLFEM_ERR_NUMERIC, "kernel evaluated outside its domain (labeled: |x - y| >= delta, or 10 labelx + labely in 14..20)");
    return NLFEM_OK;
}

// Phase event i; inside a capture it becomes an event-record node of the graph.
static cudaError_t phase_event(Session &S, int i) {
    return S.replay ? cudaEventRecordWithFlags(S.ev[i], S.st, cudaEventRecordExternal) : cudaEventRecord(S.ev[i], S.st);
}

// The assembly as one ordered sequence of stream work (also what a graph captures).
template <int DIM>
static int run_system_body(Session &S) {
    int r;
    S.nlaunch = 0;
    CK(phase_event(S, 0));
    if ((r = run_prep<DIM>(S))) return r;
    if ((r = run_dual<DIM>(S))) return r;
    if ((r = run_bfs<DIM>(S))) return r;
    if ((r = run_pairs<DIM>(S))) return r;
    if (S.pmode == PM_COLORED && (r = run_color(S))) return r;   // the one-sided passes need no colors
    if (S.dg && (r = dg_swap_in(S))) return r;   // rows: element DOFs; the search used the vertices
    CK(phase_event(S, 1));
    if ((r = run_pattern<DIM>(S))) return r;
    CK(phase_event(S, 2));
    if ((r = run_passes<DIM>(S))) return r;
    CK(phase_event(S, 3));
    if ((r = run_finish(S))) return r;
    CK(phase_event(S, 4));
    return NLFEM_OK;
}

// After the sequence: errors, timings (CUDA events on the assembly stream) and counters.
static int run_system_post(Session &S) {
    int r;
    CK(cudaStreamSynchronize(S.st));
    if ((r = check_errors(S))) return r;
    float t[4];
    for (int i = 0; i < 4; i++) CK(cudaEventElapsedTime(&t[i], S.ev[i], S.ev[i + 1]));
    unsigned long long ncl[7] = {0, 0, 0, 0, 0, 0, 0};
    if ((r = d2h(S, ncl, S.counters.get<unsigned long long>() + 4, 4))) return r;
    if ((r = d2h(S, &ncl[4], S.counters.get<unsigned long long>() + 1, 1))) return r;
    if ((r = d2h(S, &ncl[5], S.counters.get<unsigned long long>() + 12, 2))) return r;
    S.stats.n_items_in = (long)ncl[5];
    S.stats.n_items_cut = (long)ncl[6];
    S.stats.slot_map = (S.pmode == PM_RETRI || S.pmode == PM_BARY) ? (S.use_rank ? 1 : 2) : 0;
    S.stats.n_candidates = (long)ncl[4];
    S.stats.n_close = (long)ncl[0];
    S.stats.n_subtri = (long)ncl[1];
    S.stats.n_ambiguous = (long)(ncl[2] + ncl[3]);
    S.stats.ms_bfs = t[0];
    S.stats.ms_pattern = t[1];
    S.stats.ms_quad = t[2];
    S.stats.ms_finish = t[3];
    S.stats.ms_total = t[0] + t[1] + t[2] + t[3];
    S.stats.n_launches = (long)S.nlaunch;
    {
        size_t held = 0;
        for (DevBuf *b : S.buffers()) held += b->cap;
        S.stats.dev_bytes = (long)held;
    }
    g_stats = S.stats;
    return NLFEM_OK;
}

template <int DIM>
static int run_system_t(Session &S) {
    int r = run_system_body<DIM>(S);
    return r ? r : run_system_post(S);
}

// Graph replay of a session. The first call assembles normally, which sizes every buffer, and
// then captures the same sequence without host reads into a CUDA graph; later calls launch the
// graph. Capacity flags (BFS queue or pool, fixed-point range) are checked after each replay;
// if one tripped, the graph is dropped and the assembly reruns normally. Only the one-sided
// passes are captured (the colored passes read the color count on the host).
template <int DIM>
static int run_system_graph_t(Session &S) {
    int r;
    if (S.gexec) {
        const long long launches = S.nlaunch;
        CK(cudaGraphLaunch(S.gexec, S.st));
        CK(cudaStreamSynchronize(S.st));
        int he[12];
        if ((r = d2h(S, he, S.err.get<int>(), 12))) return r;
        if (!he[0] && !he[1] && !he[5] && !he[6] && !he[10] && !he[11]) {
            S.nlaunch = launches;
            return run_system_post(S);
        }
        cudaGraphExecDestroy(S.gexec);
        S.gexec = nullptr;
    }
    if ((r = run_system_t<DIM>(S))) return r;
    if (S.pmode == PM_COLORED || S.pmode == PM_VEC) return NLFEM_OK;
    const nlfem_stats keep = S.stats;
    cudaGraph_t g = nullptr;
    CK(cudaStreamBeginCapture(S.st, cudaStreamCaptureModeThreadLocal));
    S.replay = true;
    r = run_system_body<DIM>(S);
    S.replay = false;
    const long long launches = S.nlaunch;
    const cudaError_t e = cudaStreamEndCapture(S.st, &g);
    if (!r && e != cudaSuccess) r = fail(NLFEM_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(e));
    if (!r) {
        const cudaError_t ei = cudaGraphInstantiate(&S.gexec, g, 0);
        if (ei != cudaSuccess) { S.gexec = nullptr; r = fail(NLFEM_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(ei)); }
    }
    if (g) cudaGraphDestroy(g);
    cudaGetLastError();
    S.nlaunch = launches;
    S.stats = keep;
    g_stats = keep;
    return r;
}

static int run_system(Session &S) { return S.dim == 2 ? run_system_t<2>(S) : run_system_t<3>(S); }
static int run_system_graph(Session &S) { return S.dim == 2 ? run_system_graph_t<2>(S) : run_system_graph_t<3>(S); }

template <int DIM>
static int run_forcing_t(Session &S) {
    int r;
    if ((r = run_prep<DIM>(S))) return r;
    if (S.dg && (r = dg_swap_in(S))) return r;
    const long long nV = S.nV, K = (long long)S.od * nV;
    ENS(S.facc, sizeof(unsigned long long) * 2 * (K + 1));
    ENS(S.ftiny, sizeof(unsigned) * (K + 1));
    ENS(S.fd, sizeof(double) * (K + 1));
    CK(cudaMemsetAsync(S.facc.p, 0, sizeof(unsigned long long) * 2 * (K + 1), S.st));
    CK(cudaMemsetAsync(S.ftiny.p, 0, sizeof(unsigned) * (K + 1), S.st));
    const long long *zp = S.zptr.get<long long>(), *zi = S.zidx.get<long long>();
    if (S.od == 1) {
        k_forcing<DIM><<<grid_for(S.nE, 128), 128, 0, S.st>>>(S.EC.get<double>(), S.adet.get<double>(), S.labT.get<int>(), S.T32.get<int>(), S.labV.get<int>(), S.eprob.get<int>(), S.prm.get<ProbParams>(), S.nE, S.rule, zp, zi, S.facc.get<unsigned long long>(), S.ftiny.get<unsigned>());
    } else if (S.od == 2) {
        k_forcing_vec<DIM, 2><<<grid_for(S.nE, 128), 128, 0, S.st>>>(S.EC.get<double>(), S.adet.get<double>(), S.labT.get<int>(), S.T32.get<int>(), S.labV.get<int>(), S.eprob.get<int>(), S.prm.get<ProbParams>(), S.nE, S.rule, zp, zi, S.facc.get<unsigned long long>(), S.ftiny.get<unsigned>());
    } else {
        k_forcing_vec<DIM, 3><<<grid_for(S.nE, 128), 128, 0, S.st>>>(S.EC.get<double>(), S.adet.get<double>(), S.labT.get<int>(), S.T32.get<int>(), S.labV.get<int>(), S.eprob.get<int>(), S.prm.get<ProbParams>(), S.nE, S.rule, zp, zi, S.facc.get<unsigned long long>(), S.ftiny.get<unsigned>());
    }
    ++S.nlaunch;
    k_forcing_finish<<<grid_for(K, 256), 256, 0, S.st>>>(S.facc.get<unsigned long long>(), K, S.od, S.vprob.get<int>(), S.prm.get<ProbParams>(), S.fd.get<double>()); ++S.nlaunch;
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(S.st));
    return NLFEM_OK;
}

__global__ void k_export(const long long *__restrict__ fptr, const int *__restrict__ fcols, long long r0,
                         long long nrows, long long c0, long long *__restrict__ indptr,
                         long long *__restrict__ indices) {
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long base = fptr[r0];
    if (i <= nrows) indptr[i] = fptr[r0 + i] - base;
    const long long n = fptr[r0 + nrows] - base;
    for (long long j = i; j < n; j += (long long)gridDim.x * blockDim.x) indices[j] = (long long)fcols[base + j] - c0;
}

// 32-bit CSR of problem i (nnz below 2^31): row pointers rebased to the problem, columns local.
__global__ void k_export32(const long long *__restrict__ fptr, const int *__restrict__ fcols, long long r0,
                           long long nrows, int c0, int *__restrict__ indptr, int *__restrict__ indices) {
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long base = fptr[r0];
    if (i <= nrows) indptr[i] = (int)(fptr[r0 + i] - base);
    const long long n = fptr[r0 + nrows] - base;
    for (long long j = i; j < n; j += (long long)gridDim.x * blockDim.x) indices[j] = fcols[base + j] - c0;
}

// Host blocks of the 32-bit CSR results. A result's three arrays share one block (values, then
// indices, then row pointers). Blocks are pinned, so the device-to-host copies run at the
// host link's rate, and a freed block is kept for the next result (pinning is slow); plain
// malloc serves when pinning fails.
struct HostBlock {
    size_t bytes;
    bool pinned;
};
static std::mutex g_host_mu;
static std::map<void *, HostBlock> g_host_live;                 // handed out
static std::vector<std::pair<void *, HostBlock>> g_host_free;   // kept for reuse
constexpr size_t HOST_KEEP_BYTES = (size_t)16 << 30;

static void *host_take(size_t bytes) {
    std::lock_guard<std::mutex> g(g_host_mu);
    for (size_t k = 0; k < g_host_free.size(); k++)
        if (g_host_free[k].second.bytes >= bytes && g_host_free[k].second.bytes <= 2 * bytes + (1 << 20)) {
            auto e = g_host_free[k];
            g_host_free.erase(g_host_free.begin() + k);
            g_host_live[e.first] = e.second;
            return e.first;
        }
    void *p = nullptr;
    bool pinned = cudaMallocHost(&p, bytes) == cudaSuccess;
    if (!pinned) {
        cudaGetLastError();
        p = malloc(bytes);
        if (!p) return nullptr;
    }
    g_host_live[p] = HostBlock{bytes, pinned};
    return p;
}

static void host_release(void *p, const HostBlock &b) {
    if (b.pinned) cudaFreeHost(p);
    else free(p);
}

static void host_give(void *p) {
    if (!p) return;
    std::lock_guard<std::mutex> g(g_host_mu);
    auto it = g_host_live.find(p);
    if (it == g_host_live.end()) return;
    const HostBlock b = it->second;
    g_host_live.erase(it);
    size_t kept = b.bytes;
    for (auto &e : g_host_free) kept += e.second.bytes;
    if (kept > HOST_KEEP_BYTES) { host_release(p, b); return; }
    g_host_free.push_back({p, b});
}

static void host_release_free() {
    std::lock_guard<std::mutex> g(g_host_mu);
    for (auto &e : g_host_free) host_release(e.first, e.second);
    g_host_free.clear();
}

static int download32(Session &S, int i, nlfem_csr32 *out) {
    const long long r0 = (long long)S.od * S.voff[i], nrows = (long long)S.od * (S.voff[i + 1] - S.voff[i]);
    long long b[2];
    int r = d2h(S, &b[0], S.fptr.get<long long>() + r0, 1);
    if (r) return r;
    r = d2h(S, &b[1], S.fptr.get<long long>() + r0 + nrows, 1);
    if (r) return r;
    const long long nnz = b[1] - b[0];
    if (nnz > 0x7fffffffLL || nrows > 0x7fffffffLL)
        return fail(NLFEM_ERR_UNSUPPORTED, "matrix too large for 32-bit indices");
    ENS(S.out64a, sizeof(int) * (nrows + 1));
    ENS(S.out64b, sizeof(int) * (nnz + 1));
    k_export32<<<grid_for(std::max(nrows + 1, nnz), 256), 256, 0, S.st>>>(S.fptr.get<long long>(), S.fcols.get<int>(), r0, nrows, (int)r0, S.out64a.get<int>(), S.out64b.get<int>()); ++S.nlaunch;
    CK(cudaGetLastError());
    out->K = (long)nrows;
    out->nnz = (long)nnz;
    const size_t nv = (size_t)(nnz ? nnz : 1);
    unsigned char *blk = (unsigned char *)host_take(sizeof(double) * nv + sizeof(int) * (nv + nrows + 1));
    if (!blk) {
        out->indptr = nullptr; out->indices = nullptr; out->values = nullptr;
        return fail(NLFEM_ERR_NOMEM, "host allocation failed");
    }
    out->values = (double *)blk;
    out->indices = (int *)(blk + sizeof(double) * nv);
    out->indptr = out->indices + nv;
    CK(cudaMemcpyAsync(out->indptr, S.out64a.p, sizeof(int) * (nrows + 1), cudaMemcpyDeviceToHost, S.st));
    if (nnz) {
        CK(cudaMemcpyAsync(out->indices, S.out64b.p, sizeof(int) * nnz, cudaMemcpyDeviceToHost, S.st));
        CK(cudaMemcpyAsync(out->values, S.fvals.get<double>() + b[0], sizeof(double) * nnz, cudaMemcpyDeviceToHost, S.st));
    }
    CK(cudaStreamSynchronize(S.st));
    return NLFEM_OK;
}

static int download(Session &S, int i, nlfem_csr *out) {
    const long long r0 = (long long)S.od * S.voff[i], nrows = (long long)S.od * (S.voff[i + 1] - S.voff[i]);
    long long b[2];
    int r = d2h(S, &b[0], S.fptr.get<long long>() + r0, 1);
    if (r) return r;
    r = d2h(S, &b[1], S.fptr.get<long long>() + r0 + nrows, 1);
    if (r) return r;
    const long long nnz = b[1] - b[0];
    ENS(S.out64a, sizeof(long long) * (nrows + 1));
    ENS(S.out64b, sizeof(long long) * (nnz + 1));
    k_export<<<grid_for(std::max(nrows + 1, nnz), 256), 256, 0, S.st>>>(S.fptr.get<long long>(), S.fcols.get<int>(), r0, nrows, r0, S.out64a.get<long long>(), S.out64b.get<long long>()); ++S.nlaunch;
    CK(cudaGetLastError());
    out->K = (long)nrows;
    out->nnz = (long)nnz;
    out->indptr = (long *)malloc(sizeof(long) * (nrows + 1));
    out->indices = (long *)malloc(sizeof(long) * (nnz ? nnz : 1));
    out->values = (double *)malloc(sizeof(double) * (nnz ? nnz : 1));
    if (!out->indptr || !out->indices || !out->values) {
        nlfem_csr_free(out);
        return fail(NLFEM_ERR_NOMEM, "host allocation failed");
    }
    CK(cudaMemcpyAsync(out->indptr, S.out64a.p, sizeof(long long) * (nrows + 1), cudaMemcpyDeviceToHost, S.st));
    if (nnz) {
        CK(cudaMemcpyAsync(out->indices, S.out64b.p, sizeof(long long) * nnz, cudaMemcpyDeviceToHost, S.st));
        CK(cudaMemcpyAsync(out->values, S.fvals.get<double>() + b[0], sizeof(double) * nnz, cudaMemcpyDeviceToHost, S.st));
    }
    CK(cudaStreamSynchronize(S.st));
    return NLFEM_OK;
}

static int device_ok() {
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess || n == 0) {
        cudaGetLastError();
        return fail(NLFEM_ERR_CUDA, "no CUDA device available (the library has no CPU path)");
    }
    return NLFEM_OK;
}

}  // namespace nlg

// Error reporting for the entry points compiled in other translation units (not exported).
__attribute__((visibility("hidden"))) int nlfem_fail_internal(int code, const char *msg) {
    return nlg::fail(code, msg ? msg : "");
}

// ======================================================================= C ABI
using namespace nlg;

struct nlfem_session {
    Session S;
    std::vector<nlfem_problem> probs;
};

// Device buffers of the last one-shot assembly (nlfem_stiffness_matrix / _batch), kept for the
// next one on the same device so repeated calls do not allocate: buffers only grow, and every
// stage initialises what it reads. nlfem_cache_release frees them.
namespace nlg {
static std::mutex g_cache_mu;
static Session *g_cache = nullptr;
static int g_cache_dev = -1;

static void cache_take(Session &S) {
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess) { cudaGetLastError(); return; }
    std::lock_guard<std::mutex> g(g_cache_mu);
    if (!g_cache || g_cache_dev != dev) return;
    std::vector<DevBuf *> from = g_cache->buffers(), to = S.buffers();
    for (size_t i = 0; i < to.size(); i++) std::swap(*to[i], *from[i]);
    S.hint_pat_cap = g_cache->hint_pat_cap;
    S.hint_po_cap = g_cache->hint_po_cap;
    S.hint_vp_cap = g_cache->hint_vp_cap;
    S.hint_nE = g_cache->hint_nE;
    S.hint_nV = g_cache->hint_nV;
    delete g_cache;
    g_cache = nullptr;
}

static void cache_give(Session &S) {
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess) { cudaGetLastError(); return; }
    std::lock_guard<std::mutex> g(g_cache_mu);
    if (g_cache) return;   // another call's buffers are cached already: these are freed
    g_cache = new Session();
    g_cache_dev = dev;
    std::vector<DevBuf *> from = S.buffers(), to = g_cache->buffers();
    for (size_t i = 0; i < to.size(); i++) std::swap(*to[i], *from[i]);
    g_cache->hint_pat_cap = S.pat_cap;
    g_cache->hint_po_cap = S.po_cap;
    g_cache->hint_vp_cap = S.vp_cap;
    g_cache->hint_nE = S.nE;
    g_cache->hint_nV = S.nV;
}

// ---------------------------------------------------------------- CG solve on the assembled matrix
// A_Omega u = f_Omega - A_Gamma g for problem i of a session (computeRates2D.py:47-70): rows and
// unknowns are the vertices with label > 0, g holds the Dirichlet values of the vertices with
// label < 0 (label-0 columns are left out, as the reference's masks do). Conjugate gradients in
// FP64 on the session's CSR: one warp per row for the products, dot products as fixed-grid block
// partials summed on the host in a fixed order, so the iterates are deterministic.
constexpr int SOLVE_DOT_BLOCKS = 256;

__global__ void k_solve_rhs(const long long *__restrict__ fptr, const int *__restrict__ fcols,
                            const double *__restrict__ fvals, const int *__restrict__ labV, long long r0,
                            long long n, const double *__restrict__ f, const double *__restrict__ g,
                            double *__restrict__ b) {
    const int lane = threadIdx.x & 31;
    const long long w = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (w >= n) return;
    const long long row = r0 + w;
    double s = 0.0;
    if (labV[row] > 0)
        for (long long k = fptr[row] + lane; k < fptr[row + 1]; k += 32) {
            const int c = fcols[k];
            if (labV[c] < 0) s += fvals[k] * g[c - r0];
        }
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(FULL, s, o);
    if (lane == 0) b[w] = labV[row] > 0 ? f[w] - s : 0.0;
}

__global__ void k_solve_spmv(const long long *__restrict__ fptr, const int *__restrict__ fcols,
                             const double *__restrict__ fvals, const int *__restrict__ labV, long long r0,
                             long long n, const double *__restrict__ x, double *__restrict__ y) {
    const int lane = threadIdx.x & 31;
    const long long w = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (w >= n) return;
    const long long row = r0 + w;
    double s = 0.0;
    if (labV[row] > 0)
        for (long long k = fptr[row] + lane; k < fptr[row + 1]; k += 32) {
            const int c = fcols[k];
            if (labV[c] > 0) s += fvals[k] * x[c - r0];
        }
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(FULL, s, o);
    if (lane == 0) y[w] = s;
}

__global__ void k_solve_dot(const double *__restrict__ a, const double *__restrict__ b, long long n,
                            double *__restrict__ part) {
    __shared__ double sh[256];
    double s = 0.0;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        s += a[i] * b[i];
    sh[threadIdx.x] = s;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x] = sh[0];
}

// x += alpha p, r -= alpha Ap
__global__ void k_solve_update(double alpha, const double *__restrict__ p, const double *__restrict__ Ap,
                               double *__restrict__ x, double *__restrict__ r, long long n) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        x[i] += alpha * p[i];
        r[i] -= alpha * Ap[i];
    }
}
// p = r + beta p
__global__ void k_solve_dir(double beta, const double *__restrict__ r, double *__restrict__ p, long long n) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) p[i] = r[i] + beta * p[i];
}

static int solve_dot(Session &S, const double *a, const double *b, long long n, double *out) {
    k_solve_dot<<<SOLVE_DOT_BLOCKS, 256, 0, S.st>>>(a, b, n, S.sv_part.get<double>());
    CK(cudaGetLastError());
    double part[SOLVE_DOT_BLOCKS];
    int r = d2h(S, part, S.sv_part.get<double>(), SOLVE_DOT_BLOCKS);
    if (r) return r;
    double s = 0.0;
    for (int k = 0; k < SOLVE_DOT_BLOCKS; k++) s += part[k];
    *out = s;
    return NLFEM_OK;
}

static int session_solve(Session &S, int i, const double *f, const double *g, double rtol, int maxit,
                         double *u, int *iters) {
    if (S.nnz <= 0) return fail(NLFEM_ERR_INVALID, "solve needs an assembled session");
    const long long r0 = S.voff[i], n = S.voff[i + 1] - S.voff[i];
    ENS(S.sv_vec, sizeof(double) * 7 * (n + 1));
    ENS(S.sv_part, sizeof(double) * SOLVE_DOT_BLOCKS);
    double *vf = S.sv_vec.get<double>(), *vg = vf + (n + 1), *b = vg + (n + 1), *x = b + (n + 1);
    double *rr = x + (n + 1), *p = rr + (n + 1), *Ap = p + (n + 1);
    CK(cudaMemcpyAsync(vf, f, sizeof(double) * n, cudaMemcpyHostToDevice, S.st));
    CK(cudaMemcpyAsync(vg, g, sizeof(double) * n, cudaMemcpyHostToDevice, S.st));
    CK(cudaMemsetAsync(x, 0, sizeof(double) * n, S.st));
    const long long *fp = S.fptr.get<long long>();
    const int *fc = S.fcols.get<int>(), *lab = S.labV.get<int>();
    const double *fv = S.fvals.get<double>();
    const unsigned gw = grid_for(n * 32, 256), ge = grid_for(n, 256);
    k_solve_rhs<<<gw, 256, 0, S.st>>>(fp, fc, fv, lab, r0, n, vf, vg, b);
    CK(cudaMemcpyAsync(rr, b, sizeof(double) * n, cudaMemcpyDeviceToDevice, S.st));
    CK(cudaMemcpyAsync(p, b, sizeof(double) * n, cudaMemcpyDeviceToDevice, S.st));
    double bb = 0.0, rs = 0.0;
    int r = solve_dot(S, b, b, n, &bb);
    if (r) return r;
    rs = bb;
    const double stop = rtol * rtol * bb;
    int it = 0;
    while (it < maxit && rs > stop && rs > 0.0) {
        k_solve_spmv<<<gw, 256, 0, S.st>>>(fp, fc, fv, lab, r0, n, p, Ap);
        double pAp = 0.0;
        if ((r = solve_dot(S, p, Ap, n, &pAp))) return r;
        if (!(pAp > 0.0)) return fail(NLFEM_ERR_NUMERIC, "CG breakdown: the operator is not positive definite on the search direction");
        const double alpha = rs / pAp;
        k_solve_update<<<ge, 256, 0, S.st>>>(alpha, p, Ap, x, rr, n);
        double rs2 = 0.0;
        if ((r = solve_dot(S, rr, rr, n, &rs2))) return r;
        k_solve_dir<<<ge, 256, 0, S.st>>>(rs2 / rs, rr, p, n);
        rs = rs2;
        it++;
    }
    CK(cudaGetLastError());
    std::vector<int> hl(n);
    if ((r = d2h(S, u, x, n))) return r;
    if ((r = d2h(S, hl.data(), lab + r0, n))) return r;
    for (long long k = 0; k < n; k++)
        if (hl[k] < 0) u[k] = g[k];
    if (iters) *iters = it;
    if (it >= maxit && rs > stop) return fail(NLFEM_ERR_NUMERIC, "CG did not reach the tolerance within maxit iterations");
    return NLFEM_OK;
}
}  // namespace nlg

// ---------------------------------------------------------------- autotuner
// The launch shape of the two persistent kernels of an assembly, the pair search (one warp per
// outer element) and the one-sided quadrature pass (warps over a global element counter), is the
// number of blocks per SM, at most the occupancy limit. nlfem_session_autotune times each
// candidate on the session's own workload (CUDA events of the phase, best of reps assemblies),
// keeps the fastest (on a tie within 1%, the smaller one: fewer warps need less search scratch),
// and records it per device and configuration class; later sessions of the same class start from
// the recorded shape. With NLFEM_TUNE_FILE set, the records are read from and written to that file.
static std::mutex g_tune_mu;
static std::map<std::string, int> g_tune;
static bool g_tune_loaded = false;

static std::string tune_key(const Session &S, const char *stage) {
    cudaDeviceProp prop;
    int dev = 0;
    cudaGetDevice(&dev);
    std::string name = "gpu";
    if (cudaGetDeviceProperties(&prop, dev) == cudaSuccess) name = std::string(prop.name) + "/" + std::to_string(prop.multiProcessorCount);
    else cudaGetLastError();
    int kc = 0;
    for (const ProbParams &q : S.hprm) kc |= 1 << kernel_class(q);
    for (char &c : name) if (c == ' ') c = '_';
    return name + "|" + stage + "|d" + std::to_string(S.dim) + "|m" + std::to_string(S.pmode) + "|p" +
           std::to_string(S.prec) + (S.onesided64 ? "o" : "") + "|k" + std::to_string(kc);
}

static void tune_load_locked() {
    if (g_tune_loaded) return;
    g_tune_loaded = true;
    const char *path = getenv("NLFEM_TUNE_FILE");
    if (!path || !path[0]) return;
    FILE *f = fopen(path, "r");
    if (!f) return;
    char key[512];
    int v;
    while (fscanf(f, "%511s %d", key, &v) == 2) g_tune[key] = v;
    fclose(f);
}

static void tune_save_locked() {
    const char *path = getenv("NLFEM_TUNE_FILE");
    if (!path || !path[0]) return;
    FILE *f = fopen(path, "w");
    if (!f) return;
    for (auto &e : g_tune) fprintf(f, "%s %d\n", e.first.c_str(), e.second);
    fclose(f);
}

// A new session of a configuration class that was tuned before starts from the recorded shapes.
static void tune_apply(Session &S) {
    std::lock_guard<std::mutex> g(g_tune_mu);
    tune_load_locked();
    auto b = g_tune.find(tune_key(S, "bfs"));
    if (b != g_tune.end()) S.tune_bfs = b->second;
    auto p = g_tune.find(tune_key(S, "pass"));
    if (p != g_tune.end()) S.tune_pass = p->second;
}

static int session_autotune(Session &S, int reps, nlfem_tuning *out) {
    if (reps < 1) reps = 1;
    memset(out, 0, sizeof(*out));
    if (S.gexec) { cudaGraphExecDestroy(S.gexec); S.gexec = nullptr; }   // shapes are baked into a graph
    int r;
    // the search
    int best = 0;
    double best_ms = 1e300;
    for (int b = 1; b <= 8; b++) {
        S.tune_bfs = b;
        double t = 1e300;
        for (int i = 0; i < reps; i++) {
            if ((r = run_system(S))) return r;
            t = std::min(t, S.stats.ms_bfs);
        }
        if (S.used_bfs < b) break;   // beyond the occupancy limit: the same shape as b - 1
        out->bfs_ms[b - 1] = t;
        out->bfs_candidates = b;
        if (t < best_ms * 0.99) { best_ms = t; best = b; }
    }
    S.tune_bfs = best;
    out->bfs_blocks_per_sm = best;
    // the persistent quadrature pass (one-sided modes only)
    if (S.pmode == PM_RETRI || S.pmode == PM_BARY) {
        best = 0;
        best_ms = 1e300;
        for (int b = 1; b <= 8; b++) {
            S.tune_pass = b;
            double t = 1e300;
            for (int i = 0; i < reps; i++) {
                if ((r = run_system(S))) return r;
                t = std::min(t, S.stats.ms_quad);
            }
            if (S.used_pass < b) break;
            out->pass_ms[b - 1] = t;
            out->pass_candidates = b;
            if (t < best_ms * 0.99) { best_ms = t; best = b; }
        }
        S.tune_pass = best;
        out->pass_blocks_per_sm = best;
    }
    {
        std::lock_guard<std::mutex> g(g_tune_mu);
        tune_load_locked();
        g_tune[tune_key(S, "bfs")] = S.tune_bfs;
        if (S.pmode == PM_RETRI || S.pmode == PM_BARY) g_tune[tune_key(S, "pass")] = S.tune_pass;
        tune_save_locked();
    }
    return run_system(S);   // the session's matrix, assembled with the chosen shapes
}

extern "C" {

const char *nlfem_last_error(void) { return g_err.c_str(); }

int nlfem_device_count(void) {
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess) { cudaGetLastError(); return 0; }
    return n;
}

int nlfem_get_stats(nlfem_stats *out) {
    if (!out) return NLFEM_ERR_INVALID;
    *out = g_stats;
    return NLFEM_OK;
}

void nlfem_csr_free(nlfem_csr *m) {
    if (!m) return;
    free(m->indptr); free(m->indices); free(m->values);
    m->indptr = nullptr; m->indices = nullptr; m->values = nullptr;
}

void nlfem_csr32_free(nlfem_csr32 *m) {
    if (!m) return;
    host_give(m->values);   // the block holding all three arrays
    m->indptr = nullptr; m->indices = nullptr; m->values = nullptr;
}

int nlfem_session_download32(nlfem_session *s, int i, nlfem_csr32 *out) {
    if (!s || !out || i < 0 || i >= s->S.nProb) return fail(NLFEM_ERR_INVALID, "bad session download");
    return download32(s->S, i, out);
}

int nlfem_session_create(const nlfem_problem *probs, int n, nlfem_session **out) {
    if (!probs || n <= 0 || !out) return fail(NLFEM_ERR_INVALID, "no problems");
    nlfem_session *s = new nlfem_session();
    s->probs.assign(probs, probs + n);
    int r = session_init(s->S, probs, n, true);
    if (!r) tune_apply(s->S);
    if (!r) r = session_upload(s->S, probs);
    if (!r) { cudaError_t e = cudaStreamSynchronize(s->S.st); if (e != cudaSuccess) r = fail(NLFEM_ERR_CUDA, cudaGetErrorString(e)); }
    if (r) { delete s; return r; }
    *out = s;
    return NLFEM_OK;
}

int nlfem_session_assemble(nlfem_session *s) {
    if (!s) return fail(NLFEM_ERR_INVALID, "null session");
    return run_system(s->S);
}

int nlfem_session_autotune(nlfem_session *s, int reps, nlfem_tuning *out) {
    if (!s || !out) return fail(NLFEM_ERR_INVALID, "null argument");
    return session_autotune(s->S, reps, out);
}

int nlfem_session_assemble_graph(nlfem_session *s) {
    if (!s) return fail(NLFEM_ERR_INVALID, "null session");
    return run_system_graph(s->S);
}

int nlfem_session_solve(nlfem_session *s, int i, const double *f, const double *g, double rtol, int maxit,
                        double *u, int *iterations) {
    if (!s || !f || !g || !u || i < 0 || i >= s->S.nProb || !(rtol > 0.0) || maxit < 0)
        return fail(NLFEM_ERR_INVALID, "bad session solve");
    if (s->S.dg) return fail(NLFEM_ERR_UNSUPPORTED, "the solve splits rows by vertex labels: CG sessions only");
    return session_solve(s->S, i, f, g, rtol, maxit, u, iterations);
}

int nlfem_session_download(nlfem_session *s, int i, nlfem_csr *out) {
    if (!s || !out || i < 0 || i >= s->S.nProb) return fail(NLFEM_ERR_INVALID, "bad session download");
    return download(s->S, i, out);
}

void nlfem_session_destroy(nlfem_session *s) { delete s; }

int nlfem_session_set_search_epoch(nlfem_session *s, unsigned epoch) {
    if (!s) return fail(NLFEM_ERR_INVALID, "null session");
    Session &S = s->S;
    const long long nw = S.stamp_layout[0];
    if (nw <= 0) return fail(NLFEM_ERR_INVALID, "no pair search has run in this session");
    std::vector<unsigned> h((size_t)nw, epoch & 0xffffu);
    CK(cudaMemcpyAsync(S.stamp_epoch.p, h.data(), sizeof(unsigned) * (size_t)nw, cudaMemcpyHostToDevice, S.st));
    CK(cudaStreamSynchronize(S.st));
    return NLFEM_OK;
}

// One-shot session on the cached buffers of the previous one-shot call.
static int session_create_cached(const nlfem_problem *probs, int n, nlfem_session **out) {
    if (!probs || n <= 0 || !out) return fail(NLFEM_ERR_INVALID, "no problems");
    nlfem_session *s = new nlfem_session();
    cache_take(s->S);
    s->probs.assign(probs, probs + n);
    int r = session_init(s->S, probs, n, true);
    if (!r) r = session_upload(s->S, probs);
    if (r) { cache_give(s->S); delete s; return r; }
    *out = s;
    return NLFEM_OK;
}

static void session_destroy_cached(nlfem_session *s) {
    if (!s) return;
    cudaStreamSynchronize(s->S.st);
    cudaGetLastError();
    cache_give(s->S);
    delete s;
}

int nlfem_stiffness_batch(const nlfem_problem *probs, int n, nlfem_csr *outs) {
    if (!outs) return fail(NLFEM_ERR_INVALID, "null output");
    nlfem_session *s = nullptr;
    int r = session_create_cached(probs, n, &s);
    if (r) return r;
    r = run_system(s->S);
    for (int i = 0; !r && i < n; i++) r = download(s->S, i, &outs[i]);
    session_destroy_cached(s);
    return r;
}

int nlfem_stiffness_batch32(const nlfem_problem *probs, int n, nlfem_csr32 *outs) {
    if (!outs) return fail(NLFEM_ERR_INVALID, "null output");
    nlfem_session *s = nullptr;
    int r = session_create_cached(probs, n, &s);
    if (r) return r;
    r = run_system(s->S);
    for (int i = 0; !r && i < n; i++) r = download32(s->S, i, &outs[i]);
    if (r)
        for (int i = 0; i < n; i++) nlfem_csr32_free(&outs[i]);
    session_destroy_cached(s);
    return r;
}

int nlfem_stiffness_matrix32(const nlfem_problem *prob, nlfem_csr32 *out) {
    return nlfem_stiffness_batch32(prob, 1, out);
}

void nlfem_cache_release(void) {
    {
        std::lock_guard<std::mutex> g(g_cache_mu);
        delete g_cache;
        g_cache = nullptr;
    }
    host_release_free();
}

int nlfem_stiffness_matrix(const nlfem_problem *prob, nlfem_csr *out) {
    return nlfem_stiffness_batch(prob, 1, out);
}

int nlfem_load_vector(const nlfem_problem *prob, double *fd) {
    if (!prob || !fd) return fail(NLFEM_ERR_INVALID, "null argument");
    Session S;
    int r = session_init(S, prob, 1, false);
    if (!r) r = session_upload(S, prob);
    if (!r) r = (S.dim == 2) ? run_forcing_t<2>(S) : run_forcing_t<3>(S);
    if (!r) r = d2h(S, fd, S.fd.get<double>(), (size_t)S.od * S.nV);
    return r;
}

int nlfem_pair_list(const nlfem_problem *prob, long *n_pairs, long **pairs) {
    if (!prob || !n_pairs || !pairs) return fail(NLFEM_ERR_INVALID, "null argument");
    nlfem_session *s = nullptr;
    int r = nlfem_session_create(prob, 1, &s);
    if (r) return r;
    Session &S = s->S;
    S.want_pair_arrays = true;
    r = S.dim == 2 ? (run_prep<2>(S) || run_dual<2>(S) || run_bfs<2>(S) || run_pairs<2>(S))
                   : (run_prep<3>(S) || run_dual<3>(S) || run_bfs<3>(S) || run_pairs<3>(S));
    if (r) { r = g_err.empty() ? NLFEM_ERR_CUDA : r; nlfem_session_destroy(s); return r ? r : NLFEM_ERR_CUDA; }
    const long long P = S.P;
    std::vector<int> a(P), b(P);
    if (P) {
        r = d2h(S, a.data(), S.pA.get<int>(), P);
        if (!r) r = d2h(S, b.data(), S.pB.get<int>(), P);
    }
    nlfem_session_destroy(s);
    if (r) return r;
    std::vector<long long> key(P);
    for (long long i = 0; i < P; i++) key[i] = ((long long)a[i] << 32) | (unsigned)b[i];
    std::sort(key.begin(), key.end());
    long *o = (long *)malloc(sizeof(long) * 2 * (P ? P : 1));
    for (long long i = 0; i < P; i++) { o[2 * i] = (long)(key[i] >> 32); o[2 * i + 1] = (long)(key[i] & 0xffffffffLL); }
    *n_pairs = (long)P;
    *pairs = o;
    return NLFEM_OK;
}

int nlfem_pair_blocks(const nlfem_problem *prob, long n, const long *pairs, int close,
                      double *out, int *does_interact) {
    if (!prob || n < 0 || (n && (!pairs || !out || !does_interact))) return fail(NLFEM_ERR_INVALID, "null argument");
    if (n == 0) return NLFEM_OK;
    nlfem_session *s = nullptr;
    int r = nlfem_session_create(prob, 1, &s);
    if (r) return r;
    r = s->S.dim == 2 ? run_pair_blocks<2>(s->S, n, pairs, close, out, does_interact)
                      : run_pair_blocks<3>(s->S, n, pairs, close, out, does_interact);
    nlfem_session_destroy(s);
    return r;
}

int nlfem_retriangulate_batch(long n, const double *x_center, const double *TE, double sqdelta,
                              int caps, int *counts, double *out) {
    if (n < 0 || (n && (!x_center || !TE || !counts || !out))) return fail(NLFEM_ERR_INVALID, "null argument");
    if (n == 0) return NLFEM_OK;
    int r = device_ok();
    if (r) return r;
    double *dx = nullptr, *dT = nullptr, *dO = nullptr;
    int *dc = nullptr;
    CK(cudaMalloc(&dx, sizeof(double) * 2 * n));
    CK(cudaMalloc(&dT, sizeof(double) * 6 * n));
    CK(cudaMalloc(&dO, sizeof(double) * 54 * n));
    CK(cudaMalloc(&dc, sizeof(int) * n));
    CK(cudaMemcpy(dx, x_center, sizeof(double) * 2 * n, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(dT, TE, sizeof(double) * 6 * n, cudaMemcpyHostToDevice));
    CK(cudaMemset(dO, 0, sizeof(double) * 54 * n));
    k_retri_batch<<<grid_for(n, 128), 128>>>(n, dx, dT, sqdelta, caps, dc, dO);
    CK(cudaGetLastError());
    CK(cudaMemcpy(counts, dc, sizeof(int) * n, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(out, dO, sizeof(double) * 54 * n, cudaMemcpyDeviceToHost));
    cudaFree(dx); cudaFree(dT); cudaFree(dO); cudaFree(dc);
    return NLFEM_OK;
}

int nlfem_retriangulate_certified_batch(long n, const double *x_center, const double *TE, double sqdelta,
                                        int caps, int *counts, int *ambiguous, double *points) {
    if (n < 0 || (n && (!x_center || !TE || !counts || !ambiguous || !points))) return fail(NLFEM_ERR_INVALID, "null argument");
    if (n == 0) return NLFEM_OK;
    int r = device_ok();
    if (r) return r;
    double *dx = nullptr, *dT = nullptr, *dO = nullptr;
    int *dc = nullptr, *da = nullptr;
    CK(cudaMalloc(&dx, sizeof(double) * 2 * n));
    CK(cudaMalloc(&dT, sizeof(double) * 6 * n));
    CK(cudaMalloc(&dO, sizeof(double) * 18 * n));
    CK(cudaMalloc(&dc, sizeof(int) * n));
    CK(cudaMalloc(&da, sizeof(int) * n));
    CK(cudaMemcpy(dx, x_center, sizeof(double) * 2 * n, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(dT, TE, sizeof(double) * 6 * n, cudaMemcpyHostToDevice));
    CK(cudaMemset(dO, 0, sizeof(double) * 18 * n));
    k_retri_cert_batch<<<grid_for(n, 128), 128>>>(n, dx, dT, sqdelta, caps, dc, da, dO);
    CK(cudaGetLastError());
    CK(cudaMemcpy(counts, dc, sizeof(int) * n, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(ambiguous, da, sizeof(int) * n, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(points, dO, sizeof(double) * 18 * n, cudaMemcpyDeviceToHost));
    cudaFree(dx); cudaFree(dT); cudaFree(dO); cudaFree(dc); cudaFree(da);
    return NLFEM_OK;
}

int nlfem_method_retriangulate(const double *x_center, const double *TE, double sqdelta,
                               double *reTriangleList, int is_placePointOnCap) {
    int cnt = 0;
    int r = nlfem_retriangulate_batch(1, x_center, TE, sqdelta, is_placePointOnCap, &cnt, reTriangleList);
    return r ? -r : cnt;
}

static int geom_misc(int op, const double *A, int na, const double *b, int nb, int dim, double *out, int nout) {
    int r = device_ok();
    if (r) return r;
    double *dA, *db, *dO;
    int *dok, ok = 0;
    CK(cudaMalloc(&dA, sizeof(double) * na));
    CK(cudaMalloc(&db, sizeof(double) * nb));
    CK(cudaMalloc(&dO, sizeof(double) * nout));
    CK(cudaMalloc(&dok, sizeof(int)));
    CK(cudaMemcpy(dA, A, sizeof(double) * na, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(db, b, sizeof(double) * nb, cudaMemcpyHostToDevice));
    k_geom_misc<<<1, 32>>>(op, dA, db, dim, dO, dok);
    CK(cudaGetLastError());
    CK(cudaMemcpy(out, dO, sizeof(double) * nout, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(&ok, dok, sizeof(int), cudaMemcpyDeviceToHost));
    cudaFree(dA); cudaFree(db); cudaFree(dO); cudaFree(dok);
    return ok ? NLFEM_OK : fail(NLFEM_ERR_NUMERIC, "in solve2x2. Matrix not invertible.");
}

int nlfem_toRef(const double *E, const double *phys_x, double *ref_p) {
    if (!E || !phys_x || !ref_p) return fail(NLFEM_ERR_INVALID, "null argument");
    return geom_misc(0, E, 6, phys_x, 2, 2, ref_p, 2);
}
int nlfem_toPhys(const double *E, const double *p, int dim, double *out_x) {
    if (!E || !p || !out_x || (dim != 2 && dim != 3)) return fail(NLFEM_ERR_INVALID, "bad argument");
    return geom_misc(1, E, dim * (dim + 1), p, dim, dim, out_x, dim);
}
int nlfem_solve2x2(const double *A, const double *b, double *x) {
    if (!A || !b || !x) return fail(NLFEM_ERR_INVALID, "null argument");
    return geom_misc(2, A, 4, b, 2, 2, x, 2);
}

}  // extern "C"
