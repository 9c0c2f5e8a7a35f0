// Mixed-precision 2D retriangulate pass: one-sided, work-compacted, fixed-point scatter.
//
// One warp per outer element T (taken from a global work counter, so no coloring is needed).
// For each batch of 32 interacting pairs (T, b), every lane classifies its pair's outer points
// (ball contains b / misses it / cuts it); the (pair, outer point) items are compacted into an
// "inside" list and a "cut" list and processed 32 at a time, each item writing its inner sums to
// its own shared-memory slot; the owning lane then folds the slots into the pair's blocks in a
// fixed order (integrate_retriangulate, integration.cpp:345-540):
//   termLocal L (T x T), termNonloc N (T x b), termLocalPrime LP (b x b).
// All kernels of this path are functions of |x - y|, so k(y, x) = k(x, y) and
// termNonlocPrime = termNonloc exactly; the pair therefore contributes
//   A[T, T] += L,  A[T, b] -= N,  A[b, T] -= N^T,  A[b, b] += LP
// (Cassemble.cpp:737-766) and the inner element's side of the pair needs no second geometry.
// Close pairs of the singular kernel take their four FP64 blocks from closebuf instead.
// Contributions are added to the CSR values as 64-bit fixed-point integers (slots.cuh), so the
// matrix does not depend on the order in which warps finish.
//
// The pass is written once for its arithmetic type R. R = float is the mixed path: certified FP32
// geometry with the exact FP64 routine as fallback, FP32 quadrature and folds. R = double runs the
// same algorithm (same work split, classes, closed forms and fixed-point scatter) in FP64: classes
// by FP64 tests with a 2^-40 margin, every cut polygon from the exact FP64 routine (the reference's
// own), FP64 sums. Comparing the two isolates what the precision alone costs.
#pragma once
#include "passes.cuh"
#include "slots.cuh"

namespace nlg {

struct D2 {
    double x, y;
};
__device__ __forceinline__ D2 operator-(D2 a, D2 b) { return D2{a.x - b.x, a.y - b.y}; }
__device__ __forceinline__ D2 operator+(D2 a, D2 b) { return D2{a.x + b.x, a.y + b.y}; }
__device__ __forceinline__ double dot(D2 a, D2 b) { return fma(a.x, b.x, a.y * b.y); }

// Arithmetic of the pass in type R: the 2-vector type, fused multiply-add, and the FP32 or FP64
// forms of the kernel, the class test, the cut polygon and the fixed-point conversion.
template <typename R> struct Ar;
template <> struct Ar<float> {
    typedef F2 V;
    static __device__ __forceinline__ V v(float x, float y) { return F2{x, y}; }
    static __device__ __forceinline__ float fm(float a, float b, float c) { return fmaf(a, b, c); }
    static __device__ __forceinline__ float ab(float a) { return fabsf(a); }
    static __device__ __forceinline__ float ker(const ProbParams &P, float z0, float z1) { return kernel_f32(P, z0, z1); }
    static __device__ __forceinline__ float kc(const ProbParams &P) { return P.kc_f; }
    static __device__ __forceinline__ float sqd(const ProbParams &P) { return P.sqdelta_f; }
    static __device__ __forceinline__ int cls(const F2 *Q, float sq) { return fclassify(Q, sq); }
    static __device__ __forceinline__ int poly(const F2 *Q, const ProbParams &P, const double *x64, const double *E64,
                                               F2 *Rp, unsigned &namb) {
        return cut_polygon(Q, P.sqdelta_f, P, x64, E64, Rp, namb);
    }
    static __device__ __forceinline__ long long fx(float v, const ProbParams &P, bool &bad) { return fx64(v, P.fx_mul, bad); }
    static __device__ __forceinline__ const float *py(const Rule &r) { return r.Pyf; }
    static __device__ __forceinline__ const float *dy(const Rule &r) { return r.dyf; }
};

constexpr double MARG_D64 = 1.0 / 1099511627776.0;   // 2^-40, far above FP64 rounding of the tests

__device__ __forceinline__ bool dseg_far(D2 p, D2 q, double lim) {
    const D2 u = q - p;
    const double uu = dot(u, u), pu = dot(p, u);
    if (!(pu < 0.0 && -pu < uu)) return true;   // the closest point is an end point
    const double cr = fma(p.x, u.y, -p.y * u.x);
    return cr * cr > lim * uu;
}

template <> struct Ar<double> {
    typedef D2 V;
    static __device__ __forceinline__ V v(double x, double y) { return D2{x, y}; }
    static __device__ __forceinline__ double fm(double a, double b, double c) { return fma(a, b, c); }
    static __device__ __forceinline__ double ab(double a) { return fabs(a); }
    static __device__ __forceinline__ double ker(const ProbParams &P, double z0, double z1) {
        switch (P.kernel) {
        case KER_PARABOLA: return P.kc * (P.sqdelta - (z0 * z0 + z1 * z1));
        case KER_FRACTIONAL: return P.kc * exp2(-0.5 * P.expo * log2(z0 * z0 + z1 * z1));
        default: return P.kc;
        }
    }
    static __device__ __forceinline__ double kc(const ProbParams &P) { return P.kc; }
    static __device__ __forceinline__ double sqd(const ProbParams &P) { return P.sqdelta; }
    // IN and OUT only with a margin of 2^-40; everything else goes to the exact polygon
    static __device__ __forceinline__ int cls(const D2 *Q, double sq) {
        const double sqlo = sq * (1.0 - MARG_D64), sqhi = sq * (1.0 + MARG_D64);
        const double d0 = dot(Q[0], Q[0]), d1 = dot(Q[1], Q[1]), d2 = dot(Q[2], Q[2]);
        if (d0 < sqlo && d1 < sqlo && d2 < sqlo) return CLS_IN;
        if (fmin(fmin(d0, d1), d2) > sqhi && dseg_far(Q[0], Q[1], sqhi) && dseg_far(Q[1], Q[2], sqhi) &&
            dseg_far(Q[2], Q[0], sqhi))
            return CLS_OUT;
        return CLS_CUT;
    }
    // the reference's polygon (exact FP64 routine), relative to the ball center
    static __device__ __forceinline__ int poly(const D2 *, const ProbParams &P, const double *x64, const double *E64,
                                               D2 *Rp, unsigned &) {
        double R64[18];
        const int n = xretriangulate(x64, E64, P.sqdelta, P.caps, R64);
        for (int j = 0; j < n; j++) Rp[j] = D2{R64[2 * j] - x64[0], R64[2 * j + 1] - x64[1]};
        return n;
    }
    static __device__ __forceinline__ long long fx(double v, const ProbParams &P, bool &bad) {
        return fx64d(v, (double)P.fx_mul, bad);
    }
    static __device__ __forceinline__ const double *py(const Rule &r) { return r.Py; }
    static __device__ __forceinline__ const double *dy(const Rule &r) { return r.dy; }
};

constexpr int MIX_WARPS = 4;
constexpr int MIX_THREADS = 32 * MIX_WARPS;
constexpr int RES_N = 10;   // per item: innerLocal, innerNonloc[3], inner termLocalPrime sums[6]
constexpr int SCAT_U = 1;   // slot lookups per lane whose first accesses are issued together (more
                            // unrolling overflows the instruction cache of this kernel)

// Per-warp shared scratch; nPx-dependent arrays follow the struct in dynamic shared memory:
// the outer points of T (FP64, exact; FP32 relative to T's vertex 0), the item results and the
// item lists.
template <typename R>
struct MixWarp {
    R pc[32][6];            // partner element, local coordinates
    R prt[32];              // partner |det|
    int pid[32];            // partner element
    long long rhb[3], rrb[3];   // T's rows: slot map start, CSR row start
    unsigned rmask[3];          // T's rows: slot map size field (0xffffffff: no row), see RowHash
    int rlo[3];                 // T's rows: first window word (window-rank map)
    int tvs[3];                 // T's vertices
};
// One column group of a batch: the partner vertex and the integer sums of its three rows
// (termNonloc into A[T, v], termNonlocPrime into A[v, T]). Stored over the item results.
struct ScatEntry {
    int col, pad;
    long long v[6];
};
template <typename R>
__host__ __device__ constexpr size_t mix_res_bytes(int nPx) {
    return (size_t)32 * nPx * RES_N * sizeof(R) > 96 * sizeof(ScatEntry) ? (size_t)32 * nPx * RES_N * sizeof(R)
                                                                          : 96 * sizeof(ScatEntry);
}
template <typename R>
__host__ __device__ constexpr size_t mix_warp_bytes(int nPx) {
    // MixWarp + x64[nPx * 2] doubles + xf[nPx] 2-vectors + res[32][nPx][RES_N] (or the scatter
    // list) + lists[2][32 * nPx] shorts
    return ((sizeof(MixWarp<R>) + 15) / 16) * 16 + (size_t)nPx * 16 + ((size_t)nPx * 2 * sizeof(R) + 15) / 16 * 16 +
           mix_res_bytes<R>(nPx) + (size_t)2 * 32 * nPx * 2 + 16;
}


struct MixArgs {
    PassArgs p;
    SlotMap m;
    int *work;   // global element counter
    // one-sided retriangulate pass only:
    long long *valsN;   // termNonloc of each outer element into its own rows; the transposed
                        // contributions come from k_sym_add (the matrix is symmetric)
    long long *elp;     // termLocalPrime per partner element, upper triangle (k_elem_blocks adds
                        // it to the diagonal-block slots)
};

// Inner sums of one "inside" item: the ball around x contains the partner element b.
template <typename R>
__device__ __forceinline__ void item_in(const ProbParams &P, const Rule &rule, const PassRuleT<R> &pr,
                                        const R *pc, R rT, typename Ar<R>::V x, R *res) {
    typedef Ar<R> A;
    const R *Py = A::py(rule), *dy = A::dy(rule);
    const typename A::V p0 = A::v(pc[0] - x.x, pc[1] - x.y);
    const typename A::V e1 = A::v(pc[2] - pc[0], pc[3] - pc[1]), e2 = A::v(pc[4] - pc[0], pc[5] - pc[1]);
    R iL = 0, i0 = 0, i1 = 0, i2 = 0;
    R lp[6] = {0, 0, 0, 0, 0, 0};
    for (int i = 0; i < rule.nPy; i++) {
        const R px = Py[2 * i], py = Py[2 * i + 1];
        const R yx = p0.x + e1.x * px + e2.x * py;
        const R yy = p0.y + e1.y * px + e2.y * py;
        const R kw = A::ker(P, -yx, -yy) * rT;
        iL = A::fm(kw, dy[i], iL);
        i0 = A::fm(kw, pr.cy[3 * i + 0], i0);
        i1 = A::fm(kw, pr.cy[3 * i + 1], i1);
        i2 = A::fm(kw, pr.cy[3 * i + 2], i2);
#pragma unroll
        for (int ab = 0; ab < 6; ab++) lp[ab] = A::fm(kw, pr.cyy[6 * i + ab], lp[ab]);
    }
    res[0] = iL; res[1] = i0; res[2] = i1; res[3] = i2;
#pragma unroll
    for (int ab = 0; ab < 6; ab++) res[4 + ab] = lp[ab];
}

// Inner sums of one "cut" item: polygon of B(x) and b (certified FP32 with the exact FP64
// fallback, or the exact FP64 routine), fan sub-triangles, basis of b by the inverse affine map.
template <typename R>
__device__ __forceinline__ void item_cut(const ProbParams &P, const Rule &rule, const R *pc, typename Ar<R>::V x,
                                         const double *x64, const double *Eb64, R *res,
                                         unsigned &nsub, unsigned &namb) {
    typedef Ar<R> A;
    typedef typename A::V V;
    const R *Py = A::py(rule), *dy = A::dy(rule);
    const V Q[3] = {A::v(pc[0] - x.x, pc[1] - x.y), A::v(pc[2] - x.x, pc[3] - x.y), A::v(pc[4] - x.x, pc[5] - x.y)};
    const V e1 = Q[1] - Q[0], e2 = Q[2] - Q[0];
    const R idet = R(1) / (e1.x * e2.y - e1.y * e2.x);
    V Rp[9];
    const int n = A::poly(Q, P, x64, Eb64, Rp, namb);
    R iL = 0, i0 = 0, i1 = 0, i2 = 0;
    R lp[6] = {0, 0, 0, 0, 0, 0};
    for (int r = 0; r + 2 < n; r++) {
        nsub++;
        const V Av = Rp[0], B = Rp[r + 1] - Rp[0], C = Rp[r + 2] - Rp[0];
        const R rT = A::ab(B.x * C.y - B.y * C.x);
        for (int i = 0; i < rule.nPy; i++) {
            const R px = Py[2 * i], py = Py[2 * i + 1];
            const R yx = Av.x + B.x * px + C.x * py;
            const R yy = Av.y + B.y * px + C.y * py;
            const R kw = A::ker(P, -yx, -yy) * rT * dy[i];
            const R dxr = yx - Q[0].x, dyr = yy - Q[0].y;
            const R r0 = (e2.y * dxr - e2.x * dyr) * idet;
            const R r1 = (e1.x * dyr - e1.y * dxr) * idet;
            const R s0 = R(1) - r0 - r1;
            iL += kw;
            i0 = A::fm(kw, s0, i0);
            i1 = A::fm(kw, r0, i1);
            i2 = A::fm(kw, r1, i2);
            lp[0] = A::fm(kw, s0 * s0, lp[0]); lp[1] = A::fm(kw, s0 * r0, lp[1]);
            lp[2] = A::fm(kw, s0 * r1, lp[2]); lp[3] = A::fm(kw, r0 * r0, lp[3]);
            lp[4] = A::fm(kw, r0 * r1, lp[4]); lp[5] = A::fm(kw, r1 * r1, lp[5]);
        }
    }
    res[0] = iL; res[1] = i0; res[2] = i1; res[3] = i2;
#pragma unroll
    for (int ab = 0; ab < 6; ab++) res[4 + ab] = lp[ab];
}

// Inner sums of one "cut" item for a constant kernel. The kernel weight of every inner point is
// kc |S| dy_i, and the basis functions of b are affine, so on a fan sub-triangle S = (A, B, C)
// psi_a(y_i) = psi_a(A) + (psi_a(B) - psi_a(A)) px_i + (psi_a(C) - psi_a(A)) py_i, and the rule's
// sums over S follow from its moments m = sum_i dy_i (1, px, py, px^2, px py, py^2):
//   sum_i dy_i psi_a = al_a m0 + be_a mx + ga_a my,
//   sum_i dy_i psi_a psi_b = al_a t0_b + be_a t1_b + ga_a t2_b  (t_b the first sums of psi_b with
//   weights (1, px, py)).
// This equals the quadrature sum of the general item for any rule. The basis values come from the
// polygon's points (one evaluation per point instead of per inner point), and every sum stays in
// the basis functions' own range, so no cancellation enters where a basis function is small.
template <typename R>
__device__ __forceinline__ void item_cut_const(const ProbParams &P, const PassRuleT<R> &pr, const R *pc,
                                               typename Ar<R>::V x, const double *x64, const double *Eb64, R *res,
                                               unsigned &nsub, unsigned &namb) {
    typedef Ar<R> A;
    typedef typename A::V V;
    const V Q[3] = {A::v(pc[0] - x.x, pc[1] - x.y), A::v(pc[2] - x.x, pc[3] - x.y), A::v(pc[4] - x.x, pc[5] - x.y)};
    const V e1 = Q[1] - Q[0], e2 = Q[2] - Q[0];
    const R idet = R(1) / (e1.x * e2.y - e1.y * e2.x);
    V Rp[9];
    const int n = A::poly(Q, P, x64, Eb64, Rp, namb);
    const R m0 = pr.mom[0], mx = pr.mom[1], my = pr.mom[2], mxx = pr.mom[3], mxy = pr.mom[4], myy = pr.mom[5];
    auto basis = [&](V y, R *l) {   // psi_0..2 of b at y (as the general item evaluates them)
        const R dxr = y.x - Q[0].x, dyr = y.y - Q[0].y;
        l[1] = (e2.y * dxr - e2.x * dyr) * idet;
        l[2] = (e1.x * dyr - e1.y * dxr) * idet;
        l[0] = R(1) - l[1] - l[2];
    };
    R S0 = 0, S1[3] = {0, 0, 0}, S2[6] = {0, 0, 0, 0, 0, 0};
    R la[3], lb[3], lc[3];
    if (n >= 3) {
        basis(Rp[0], la);
        basis(Rp[1], lb);
    }
    for (int r = 0; r + 2 < n; r++) {
        nsub++;
        const V B = Rp[r + 1] - Rp[0], C = Rp[r + 2] - Rp[0];
        const R rT = A::ab(B.x * C.y - B.y * C.x);
        basis(Rp[r + 2], lc);
        R t0[3], t1[3], t2[3];
#pragma unroll
        for (int q = 0; q < 3; q++) {
            const R al = la[q], be = lb[q] - la[q], ga = lc[q] - la[q];
            t0[q] = A::fm(al, m0, A::fm(be, mx, ga * my));
            t1[q] = A::fm(al, mx, A::fm(be, mxx, ga * mxy));
            t2[q] = A::fm(al, my, A::fm(be, mxy, ga * myy));
        }
        S0 = A::fm(rT, m0, S0);
        int t = 0;
#pragma unroll
        for (int q = 0; q < 3; q++) {
            S1[q] = A::fm(rT, t0[q], S1[q]);
            const R al = la[q], be = lb[q] - la[q], ga = lc[q] - la[q];
#pragma unroll
            for (int q2 = q; q2 < 3; q2++, t++) S2[t] = A::fm(rT, A::fm(al, t0[q2], A::fm(be, t1[q2], ga * t2[q2])), S2[t]);
        }
#pragma unroll
        for (int q = 0; q < 3; q++) lb[q] = lc[q];
    }
    const R kc = A::kc(P);
    res[0] = kc * S0;
#pragma unroll
    for (int q = 0; q < 3; q++) res[1 + q] = kc * S1[q];
#pragma unroll
    for (int q = 0; q < 6; q++) res[4 + q] = kc * S2[q];
}

// Appends this lane's items of class cls (one per outer point k with that class) to list, in
// (k, lane) order; returns the list length (uniform).
__device__ __forceinline__ int build_list(const unsigned char *mycls, int nPx, int cls,
                                          unsigned short *list) {
    const int lane = threadIdx.x & 31;
    int n = 0;
    for (int k = 0; k < nPx; k++) {
        const bool mine = mycls[k] == cls;
        const unsigned m = __ballot_sync(FULL, mine);
        if (mine) list[n + __popc(m & lanemask_lt())] = (unsigned short)(k * 32 + lane);
        n += __popc(m);
    }
    __syncwarp();
    return n;
}

// The same from a bit mask of the lane's outer points (bit k: item (k, lane) is in the list).
__device__ __forceinline__ int build_list_mask(unsigned mask, int nPx, unsigned short *list) {
    const int lane = threadIdx.x & 31;
    int n = 0;
    for (int k = 0; k < nPx; k++) {
        const bool mine = (mask >> k) & 1u;
        const unsigned m = __ballot_sync(FULL, mine);
        if (mine) list[n + __popc(m & lanemask_lt())] = (unsigned short)(k * 32 + lane);
        n += __popc(m);
    }
    __syncwarp();
    return n;
}

// a[i] for i in {0, 1, 2} as register selects (no dynamic indexing of register arrays)
template <typename X>
__device__ __forceinline__ X sel3(const X *v, int i) {
    return i == 0 ? v[0] : (i == 1 ? v[1] : v[2]);
}

__device__ __forceinline__ long long shfl64(long long v, int src) {
    return (long long)__shfl_sync(FULL, (unsigned long long)v, src);
}

// KIND: the kernel class of the launch's problems. MIX_CONST: constant kernels; inside items take
// the rule's precomputed element sums and cut items the moment form (item_cut_const). MIX_REGULAR:
// other kernels without close pairs. MIX_SINGULAR: singular kernels whose close pairs come from
// the Duffy blocks. Each instance holds only its class's code, which keeps the kernel small (it is
// bound by instruction fetch as much as by anything else).
enum { MIX_CONST = 0, MIX_REGULAR = 1, MIX_SINGULAR = 2 };
template <int KIND, typename R>
__global__ void __launch_bounds__(MIX_THREADS, 4) k_pass_mix2d(MixArgs ma, Rule rule, PassRuleT<R> pr) {
    typedef Ar<R> A;
    typedef typename A::V V;
    constexpr bool F32 = sizeof(R) == 4;
    constexpr bool CK = KIND == MIX_CONST;
    extern __shared__ __align__(16) unsigned char s_raw[];
    const PassArgs &a = ma.p;
    const SlotMap &sm = ma.m;
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const int nPx = rule.nPx;
    unsigned char *wbase = s_raw + (size_t)wib * mix_warp_bytes<R>(nPx);
    MixWarp<R> &W = *reinterpret_cast<MixWarp<R> *>(wbase);
    double *x64 = reinterpret_cast<double *>(wbase + ((sizeof(MixWarp<R>) + 15) / 16) * 16);   // [nPx * 2]
    V *xf = reinterpret_cast<V *>(x64 + 2 * nPx);                                              // [nPx]
    R *res = reinterpret_cast<R *>(reinterpret_cast<unsigned char *>(xf) + ((size_t)nPx * 2 * sizeof(R) + 15) / 16 * 16);   // [32][nPx][RES_N]
    unsigned short *lst = reinterpret_cast<unsigned short *>(reinterpret_cast<unsigned char *>(res) + mix_res_bytes<R>(nPx));   // [2][32*nPx]
    ScatEntry *slist = reinterpret_cast<ScatEntry *>(res);   // scatter list, after the fold
    long long *vals = reinterpret_cast<long long *>(a.vals);
    int *ovf = &a.err[5];
    bool bad = false;   // a contribution outside the fixed-point range (reported at the end)
    bool miss = false;  // a matrix slot not found (reported at the end)
    unsigned nsub = 0, namb = 0, nclose = 0, nitin = 0, nitcut = 0;
    for (;;) {
        int idx = 0;
        if (lane == 0) idx = atomicAdd(ma.work, 1);
        idx = __shfl_sync(FULL, idx, 0);
        if (idx >= a.count) break;
        const int T = a.list ? a.list[idx] : idx;
        const long long lb = a.out_ptr[T], le = a.out_cnt ? lb + a.out_cnt[T] : a.out_ptr[T + 1];
        if (lb == le || a.labT[T] == 0) continue;
        int tv[3];
        unsigned keepmask = 0;   // bit r: the row of T's vertex r exists
#pragma unroll
        for (int r = 0; r < 3; r++) {
            tv[r] = a.T32[(long long)T * 3 + r];
            if (a.labV[tv[r]] > 0) keepmask |= 1u << r;
        }
        if (lane < 3) {   // T's rows, for the lookups of every batch
            const int u = sel3(tv, lane);
            RowHash h;
            h.hb = h.rb = 0;
            h.mask = 0xffffffffu;
            h.lo = 0;
            if (keepmask & (1u << lane)) h = row_hash(sm, u);
            W.rhb[lane] = h.hb;
            W.rrb[lane] = h.rb;
            W.rmask[lane] = h.mask;
            W.rlo[lane] = h.lo;
            W.tvs[lane] = u;
        }
        const ProbParams P = a.probs[a.eprob[T]];
        const double *ET64 = &a.EC[(long long)T * 6];
        const float ohi0 = a.EChi[(long long)T * 6], ohi1 = a.EChi[(long long)T * 6 + 1];
        const float olo0 = a.EClo[(long long)T * 6], olo1 = a.EClo[(long long)T * 6 + 1];
        const R rTT = F32 ? (R)a.adetf[T] : (R)a.adet[T];
        for (int k = lane; k < nPx; k += 32) {
            xtoPhys<2>(ET64, &rule.Px[2 * k], &x64[2 * k]);
            xf[k] = A::v((R)(x64[2 * k] - ET64[0]), (R)(x64[2 * k + 1] - ET64[1]));
        }
        __syncwarp();
        long long D[6];   // termLocal of T's pairs, integer sums
#pragma unroll
        for (int i = 0; i < 6; i++) D[i] = 0;
        const bool frac_close = KIND == MIX_SINGULAR && duffy_close(P);   // fractional or weakSingular close blocks
        const R sqf = A::sqd(P);
        int part_next = lb + lane < le ? a.pB[lb + lane] : T;   // partners one batch ahead
        for (long long p0 = lb; p0 < le; p0 += 32) {
            const long long p = p0 + lane;
            const bool act = p < le;
            const int part = part_next;
            part_next = p + 32 < le ? a.pB[p + 32] : T;
            int pv[3];
#pragma unroll
            for (int r = 0; r < 3; r++) pv[r] = a.T32[(long long)part * 3 + r];
            bool close = false;
            if (frac_close && act) {
                close = (part == T);
#pragma unroll
                for (int i = 0; i < 3; i++)
#pragma unroll
                    for (int j = 0; j < 3; j++) close |= (tv[i] == pv[j]);
            }
            // owner: partner data and classes
            R pc[6];
#pragma unroll
            for (int j = 0; j < 6; j++) {
                if (F32)
                    pc[j] = (a.EChi[(long long)part * 6 + j] - ((j & 1) ? ohi1 : ohi0)) + (a.EClo[(long long)part * 6 + j] - ((j & 1) ? olo1 : olo0));
                else
                    pc[j] = (R)(a.EC[(long long)part * 6 + j] - ET64[j & 1]);
            }
#pragma unroll
            for (int j = 0; j < 6; j++) W.pc[lane][j] = pc[j];
            W.prt[lane] = F32 ? (R)a.adetf[part] : (R)a.adet[part];
            W.pid[lane] = part;
            // classes as bit masks over the outer points: inm (ball contains the partner), cutm
            // (ball cuts it). Only cut items (and, for other kernels, inside items) write their
            // sums into res; the fold reads res for those items only.
            unsigned inm = 0, cutm = 0;
            for (int k = 0; k < nPx; k++) {
                int c = CLS_OUT;
                if (act && !close) {
                    const V x = xf[k];
                    const V Q[3] = {A::v(pc[0] - x.x, pc[1] - x.y), A::v(pc[2] - x.x, pc[3] - x.y), A::v(pc[4] - x.x, pc[5] - x.y)};
                    c = A::cls(Q, sqf);
                }
                inm |= (unsigned)(c == CLS_IN) << k;
                cutm |= (unsigned)(c == CLS_CUT) << k;
            }
            nitin += __popc(inm);
            nitcut += __popc(cutm);
            if (CK) nsub += __popc(inm);
            __syncwarp();
            const int nin = CK ? 0 : build_list_mask(inm, nPx, lst);
            const int ncut = build_list_mask(cutm, nPx, lst + 32 * nPx);
            for (int c0 = 0; c0 < nin; c0 += 32) {
                if (c0 + lane < nin) {
                    const int it = lst[c0 + lane];
                    const int k = it >> 5, j = it & 31;
                    nsub++;
                    item_in(P, rule, pr, W.pc[j], W.prt[j], xf[k], &res[(j * nPx + k) * RES_N]);
                }
            }
            for (int c0 = 0; c0 < ncut; c0 += 32) {
                if (c0 + lane < ncut) {
                    const int it = lst[32 * nPx + c0 + lane];
                    const int k = it >> 5, j = it & 31;
                    if (CK)
                        item_cut_const(P, pr, W.pc[j], xf[k], &x64[2 * k], &a.EC[(long long)W.pid[j] * 6],
                                       &res[(j * nPx + k) * RES_N], nsub, namb);
                    else
                        item_cut(P, rule, W.pc[j], xf[k], &x64[2 * k], &a.EC[(long long)W.pid[j] * 6],
                                 &res[(j * nPx + k) * RES_N], nsub, namb);
                }
            }
            __syncwarp();
            // owner: fold the item sums into the pair's blocks, in fixed point from here on
            long long nx[9], mx[9], lpx[6], lx[6];
#pragma unroll
            for (int i = 0; i < 9; i++) nx[i] = mx[i] = 0;
#pragma unroll
            for (int i = 0; i < 6; i++) lpx[i] = lx[i] = 0;
            // constant kernel: a pair with every outer point inside takes the precomputed sums
            // (lanefull), so its blocks do not depend on the other pairs of its batch; when that
            // holds for every active pair (a warp vote, taken here where all lanes are present)
            // the outer-point loop is skipped
            const unsigned fullm = nPx >= 32 ? 0xffffffffu : (1u << nPx) - 1u;
            const bool lanefull = CK && inm == fullm;
            const bool allin = CK && __all_sync(FULL, !act || close || lanefull);
            if (act) {
                if (close) {
                    nclose++;
                    const long long cs = close_slot(a.xadj, a.adj, T, part);
                    if (cs < 0) {
                        miss = true;
                    } else {
                        const double *cb = &a.closebuf[cs * 36];
#pragma unroll
                        for (int i = 0; i < 3; i++)
#pragma unroll
                            for (int j = i + 1; j < 3; j++) lx[sym_idx<3>(i, j)] = fx64d(cb[3 * i + j], P.fx_mul, bad);
#pragma unroll
                        for (int i = 0; i < 9; i++) {
                            nx[i] = fx64d(cb[9 + i], P.fx_mul, bad);    // termNonloc [T vertex][b vertex]
                            mx[i] = fx64d(cb[27 + i], P.fx_mul, bad);   // termNonlocPrime [T vertex][b vertex]
                        }
#pragma unroll
                        for (int i = 0; i < 3; i++)
#pragma unroll
                            for (int j = i + 1; j < 3; j++) lpx[sym_idx<3>(i, j)] = fx64d(cb[18 + 3 * i + j], P.fx_mul, bad);
                    }
                } else {
                    R L[6] = {0, 0, 0, 0, 0, 0}, N[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
                    R LP[6] = {0, 0, 0, 0, 0, 0};
                    // the outer-point loop is warp-uniform (the rule's constants are read at one
                    // address per warp); each lane adds the items its classes select
                    R Axx[6] = {0, 0, 0, 0, 0, 0}, Ax[3] = {0, 0, 0}, Ad = 0;   // inside items (constant kernel)
                    if (lanefull) {   // every item inside: the rule's sums over all outer points
#pragma unroll
                        for (int ab = 0; ab < 6; ab++) Axx[ab] = pr.xsum[ab];
#pragma unroll
                        for (int r = 0; r < 3; r++) Ax[r] = pr.xsum[6 + r];
                        Ad = pr.xsum[9];
                    }
                    if (!allin) {
                        for (int k = 0; k < nPx; k++) {
                            if (lanefull) continue;
                            if (CK && ((inm >> k) & 1u)) {
#pragma unroll
                                for (int ab = 0; ab < 6; ab++) Axx[ab] += pr.cxx[6 * k + ab];
#pragma unroll
                                for (int r = 0; r < 3; r++) Ax[r] += pr.cx[3 * k + r];
                                Ad += pr.dxf[k];
                                continue;
                            }
                            if (!(((inm | cutm) >> k) & 1u)) continue;
                            const R *rr = &res[(lane * nPx + k) * RES_N];
                            const R dk = pr.dxf[k];
#pragma unroll
                            for (int ab = 0; ab < 6; ab++) L[ab] = A::fm(pr.cxx[6 * k + ab], rr[0], L[ab]);
#pragma unroll
                            for (int r = 0; r < 3; r++) {
                                const R c = pr.cx[3 * k + r];
                                N[3 * r + 0] = A::fm(c, rr[1], N[3 * r + 0]);
                                N[3 * r + 1] = A::fm(c, rr[2], N[3 * r + 1]);
                                N[3 * r + 2] = A::fm(c, rr[3], N[3 * r + 2]);
                            }
#pragma unroll
                            for (int ab = 0; ab < 6; ab++) LP[ab] = A::fm(dk, rr[4 + ab], LP[ab]);
                        }
                    }
                    if (CK) {   // an inside item's sums are kc |b| times the rule's element sums
                        R inv[RES_N];
                        const R kr = A::kc(P) * W.prt[lane];
#pragma unroll
                        for (int q = 0; q < RES_N; q++) inv[q] = kr * pr.insum[q];
#pragma unroll
                        for (int ab = 0; ab < 6; ab++) L[ab] = A::fm(Axx[ab], inv[0], L[ab]);
#pragma unroll
                        for (int r = 0; r < 3; r++) {
                            N[3 * r + 0] = A::fm(Ax[r], inv[1], N[3 * r + 0]);
                            N[3 * r + 1] = A::fm(Ax[r], inv[2], N[3 * r + 1]);
                            N[3 * r + 2] = A::fm(Ax[r], inv[3], N[3 * r + 2]);
                        }
#pragma unroll
                        for (int ab = 0; ab < 6; ab++) LP[ab] = A::fm(Ad, inv[4 + ab], LP[ab]);
                    }
#pragma unroll
                    for (int i = 0; i < 6; i++)   // the diagonal entries come from the row sums (k_sym_add)
                        if (i != 0 && i != 3 && i != 5) lx[i] = A::fx(L[i] * rTT, P, bad);
#pragma unroll
                    for (int i = 0; i < 9; i++) mx[i] = nx[i] = A::fx(N[i] * rTT, P, bad);
#pragma unroll
                    for (int i = 0; i < 6; i++)
                        if (i != 0 && i != 3 && i != 5) lpx[i] = A::fx(LP[i] * rTT, P, bad);
                }
                // Only off-diagonal entries of the matrix are accumulated: every kept row of the
                // assembled operator sums to zero (for kernels of |x - y| each pair's blocks do, the
                // basis functions summing to one), so k_sym_add sets each diagonal entry to minus
                // its row's off-diagonal sum. The integers are those a per-pair balance of the
                // block diagonals would give, so the matrix is the same bit for bit.
#pragma unroll
                for (int i = 0; i < 6; i++) D[i] += lx[i];
                // termLocalPrime (off-diagonal part) into the partner's block accumulator
                red_add(ma.elp, (long long)part * 6 + 1, lpx[1]);
                red_add(ma.elp, (long long)part * 6 + 2, lpx[2]);
                red_add(ma.elp, (long long)part * 6 + 4, lpx[4]);
            }
            // termNonloc into A[T, b] (minus sign): lanes sharing a partner vertex add their
            // integers, the first of them lists the sums (over the item results, read by now); then
            // all lanes share the (vertex, row) lookups. The mirror A[b, T] -= N^T comes from the
            // symmetric completion (k_sym_add), except where T's vertex has no row (written here
            // into the partner vertex's row) and for close pairs, whose termNonlocPrime block is
            // its own FP64 result (the difference to N^T is added here).
            __syncwarp();
            const bool anyclose = KIND == MIX_SINGULAR && __any_sync(FULL, close);
            int nent = 0;
#pragma unroll 1
            for (int c = 0; c < 3; c++) {
                const int col = act ? sel3(pv, c) : -1;
                const unsigned grp = __match_any_sync(FULL, col);
                const bool leader = (__ffs(grp) - 1) == lane;
                const int maxn = __reduce_max_sync(FULL, (unsigned)__popc(grp));
                const long long o0 = sel3(&nx[0], c), o1 = sel3(&nx[3], c), o2 = sel3(&nx[6], c);
                const long long p0v = sel3(&mx[0], c), p1v = sel3(&mx[3], c), p2v = sel3(&mx[6], c);
                long long sn0 = o0, sn1 = o1, sn2 = o2, sq0 = p0v, sq1 = p1v, sq2 = p2v;
                unsigned rest = grp & ~(1u << lane);
                for (int it = 1; it < maxn; it++) {
                    const int src = rest ? __ffs(rest) - 1 : lane;
                    const bool use = rest != 0;
                    if (rest) rest &= rest - 1;
                    const long long t0 = shfl64(o0, src), t1 = shfl64(o1, src), t2 = shfl64(o2, src);
                    if (use) { sn0 += t0; sn1 += t1; sn2 += t2; }
                    if (anyclose) {
                        const long long u0 = shfl64(p0v, src), u1 = shfl64(p1v, src), u2 = shfl64(p2v, src);
                        if (use) { sq0 += u0; sq1 += u1; sq2 += u2; }
                    }
                }
                if (!anyclose) { sq0 = sn0; sq1 = sn1; sq2 = sn2; }
                const bool put = leader && col >= 0;
                const unsigned m = __ballot_sync(FULL, put);
                if (put) {
                    ScatEntry &e = slist[nent + __popc(m & lanemask_lt())];
                    e.col = col;
                    e.v[0] = sn0; e.v[1] = sn1; e.v[2] = sn2;
                    e.v[3] = sq0; e.v[4] = sq1; e.v[5] = sq2;
                }
                nent += __popc(m);
            }
            __syncwarp();
            // (row, column) lookups, SCAT_U per lane at a time: the first memory access of each is
            // issued before any is examined, so their latencies overlap
            const int nit = 3 * nent;
            for (int w0 = 0; w0 < nit; w0 += 32 * SCAT_U) {
                SlotProbe pb[SCAT_U];
#pragma unroll
                for (int u = 0; u < SCAT_U; u++) {
                    const int w = w0 + lane + 32 * u;
                    pb[u].e = HEMPTY;
                    pb[u].i = 0;
                    if (w < nit) {
                        const int e = w / 3, r = w - 3 * e;
                        RowHash h;
                        h.hb = W.rhb[r]; h.rb = W.rrb[r]; h.mask = W.rmask[r]; h.lo = W.rlo[r];
                        pb[u] = slot_probe_begin(sm, h, slist[e].col);
                    }
                }
#pragma unroll
                for (int u = 0; u < SCAT_U; u++) {
                    const int w = w0 + lane + 32 * u;
                    if (w >= nit) continue;
                    const int e = w / 3, r = w - 3 * e;
                    const int col = slist[e].col;
                    if (col == W.tvs[r]) continue;   // the matrix diagonal: from the row sum
                    const long long sn = slist[e].v[r], sq = slist[e].v[3 + r];
                    RowHash h;
                    h.hb = W.rhb[r]; h.rb = W.rrb[r]; h.mask = W.rmask[r]; h.lo = W.rlo[r];
                    if (h.mask != 0xffffffffu) {
                        const long long s = slot_probe_end(sm, h, col, pb[u]);
                        if (s < 0) { miss = true; continue; }
                        red_add(ma.valsN, s, -sn);
                        if (anyclose && sq != sn && a.labV[col] > 0) {
                            const int tp = sm.tpos[s];
                            if (tp < 0) miss = true;
                            else red_add(vals, sm.rowptr[col] + tp, sn - sq);
                        }
                    } else if (a.labV[col] > 0) {
                        const long long q = slot_find(sm, col, W.tvs[r]);
                        if (q < 0) miss = true;
                        else red_add(vals, q, -sq);
                    }
                }
            }
            __syncwarp();
        }
        // termLocal of all of T's pairs into T's diagonal block
#pragma unroll
        for (int i = 0; i < 6; i++)
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) D[i] += (long long)__shfl_xor_sync(FULL, (unsigned long long)D[i], o);
        if (lane < 9 && lane / 3 != lane % 3) {   // off-diagonal entries (the diagonal: k_sym_add)
            const int r = lane / 3, c = lane % 3;
            const int s = sm.dslot[(long long)T * 9 + lane];
            const int si = r <= c ? sym_idx<3>(r, c) : sym_idx<3>(c, r);
            long long d = 0;
#pragma unroll
            for (int i = 0; i < 6; i++)
                if (i == si) d = D[i];
            if (s >= 0) red_add(vals, s, d);
            else if (keepmask & (1u << r)) miss = true;
        }
        __syncwarp();
    }
    if (__any_sync(FULL, bad) && lane == 0) atomicOr(ovf, 1);
    if (__any_sync(FULL, miss) && lane == 0) atomicOr(&a.err[3], 1);
    nsub = warp_sum(nsub);
    namb = warp_sum(namb);
    nclose = warp_sum(nclose);
    nitin = warp_sum(nitin);
    nitcut = warp_sum(nitcut);
    if (lane == 0) {
        if (nsub && a.n_subtri) atomicAdd(a.n_subtri, (unsigned long long)nsub);
        if (namb && a.n_amb) atomicAdd(a.n_amb, (unsigned long long)namb);
        if (nclose && a.n_close) atomicAdd(a.n_close, (unsigned long long)nclose);
        if (nitin && a.n_in) atomicAdd(a.n_in, (unsigned long long)nitin);
        if (nitcut && a.n_cut) atomicAdd(a.n_cut, (unsigned long long)nitcut);
    }
}

// Symmetric completion of the one-sided retriangulate pass: every slot (t, v) adds the
// termNonloc sums of the transposed slot (v, t) when v has a row. Integer sums, so the completed
// matrix is exactly symmetric in these contributions, as the reference's A[b, T] -= termNonlocPrime
// = termNonloc^T (kernels of |x - y|) makes it. Then the row's diagonal entry is set to minus the
// sum of its other entries, which the pass left out (every kept row sums to zero). One warp per row.
__global__ void k_sym_add(const long long *__restrict__ rowptr, const int *__restrict__ cols,
                          const int *__restrict__ tpos, const long long *__restrict__ valsN, long long nrows,
                          long long *__restrict__ vals) {
    const int lane = threadIdx.x & 31;
    const long long gw = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const long long nw = ((long long)gridDim.x * blockDim.x) >> 5;
    for (long long t = gw; t < nrows; t += nw) {
        const long long b = rowptr[t], e = rowptr[t + 1];
        long long off = 0, dslot = -1;
        for (long long s = b + lane; s < e; s += 32) {
            if (cols[s] == (int)t) { dslot = s; continue; }
            long long v = valsN[s];
            const int tp = tpos[s];
            if (tp >= 0) v += valsN[rowptr[cols[s]] + tp];
            v += vals[s];
            vals[s] = v;
            off += v;
        }
        off = (long long)warp_sum((unsigned long long)off);
        if (dslot >= 0) vals[dslot] = -off;   // the row sums to zero
    }
}

// termLocalPrime blocks accumulated per partner element into its diagonal-block slots.
__global__ void k_elem_blocks(const long long *__restrict__ elp, const int *__restrict__ dslot,
                              const int *__restrict__ T32, const int *__restrict__ labV, long long nE,
                              long long *__restrict__ vals, int *__restrict__ err) {
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= nE) return;
    long long b[6];
    bool any = false;
#pragma unroll
    for (int q = 0; q < 6; q++) {
        b[q] = elp[e * 6 + q];
        any |= b[q] != 0;
    }
    if (!any) return;
#pragma unroll
    for (int r = 0; r < 3; r++)
#pragma unroll
        for (int c = 0; c < 3; c++) {
            if (r == c) continue;   // the diagonal comes from the row sum (k_sym_add)
            const int s = dslot[e * 9 + 3 * r + c];
            if (s >= 0) red_add(vals, s, b[r <= c ? sym_idx<3>(r, c) : sym_idx<3>(c, r)]);
            else if (labV[T32[e * 3 + r]] > 0) atomicOr(&err[3], 1);
        }
}

}  // namespace nlg
