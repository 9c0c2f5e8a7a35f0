// Element-colored assembly passes.
//
// Elements are colored so that no two elements of a color share a vertex (deterministic
// Jones-Plassmann on the vertex-sharing dual graph). One launch per color; one warp per element T
// of the color computes every contribution that lands in the rows of T's vertices:
//   out side  pairs (T, bT), bT in out(T): termLocal -> A[T, T] and termNonloc -> A[T, bT]
//   in side   pairs (aT, T), aT in in(T):  termLocalPrime -> A[T, T], termNonlocPrime -> A[T, aT]
// (src/Cassemble.cpp:721-770). No other warp of the launch touches these rows, so the warp adds
// into the FP64 CSR values directly: lanes that hit the same column are summed in lane order and
// the group's first lane performs the add. Lists are sorted and colors run in a fixed order, so
// the summation order, and hence every bit of the result, is the same on every run.
//
// Quadrature precision (template PREC):
//   PREC_F64: the reference's FP64 arithmetic, exact retriangulation for every outer point.
//   PREC_MIX: FP32 quadrature on coordinates local to T (double-float differences), certified
//             FP32 ball-triangle geometry with exact FP64 fallback, FP64 accumulation of the
//             per-element blocks and of the CSR values.
#pragma once
#include "certified.cuh"
#include "geometry.cuh"
#include "primitives.cuh"
#include "quadrature.cuh"

namespace nlg {

enum { PREC_F64 = 0, PREC_MIX = 1 };

// ---------------------------------------------------------------- coloring
__device__ __forceinline__ unsigned hash32(unsigned x) {
    x ^= x >> 16; x *= 0x7feb352dU; x ^= x >> 15; x *= 0x846ca68bU; x ^= x >> 16;
    return x;
}

// One Jones-Plassmann round: an uncolored element whose priority beats every uncolored neighbour
// takes the smallest color none of its colored neighbours has. Reads cur, writes nxt.
// Priorities hash the problem-local element index, so a problem colors the same alone or batched.
__global__ void k_color_round(const long long *__restrict__ xadj, const int *__restrict__ adj,
                              long long nE, const int *__restrict__ eprob,
                              const ProbParams *__restrict__ probs, const int *__restrict__ cur,
                              int *__restrict__ nxt, unsigned long long *__restrict__ remaining,
                              int *__restrict__ err) {
    long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= nE) return;
    const int c0 = cur[e];
    if (c0 >= 0) { nxt[e] = c0; return; }
    const int off = probs[eprob[e]].elem_off;
    const unsigned le = (unsigned)(e - off);
    const unsigned pe = hash32(le);
    unsigned long long used[4] = {0, 0, 0, 0};
    bool win = true;
    for (long long j = xadj[e]; j < xadj[e + 1]; j++) {
        const int n = adj[j];
        const int c = cur[n];
        if (c < 0) {
            const unsigned ln = (unsigned)(n - off);
            const unsigned pn = hash32(ln);
            if (pn > pe || (pn == pe && ln > le)) win = false;
        } else if (c < 256) {
            used[c >> 6] |= 1ULL << (c & 63);
        }
    }
    if (!win) { nxt[e] = -1; atomicAdd(remaining, 1ULL); return; }
    int c = -1;
    for (int w = 0; w < 4 && c < 0; w++)
        if (~used[w]) c = 64 * w + __ffsll((long long)~used[w]) - 1;
    if (c < 0) { atomicOr(err, 1); c = 0; }
    nxt[e] = c;
}

__global__ void k_color_count(const int *__restrict__ color, long long nE, int *__restrict__ cnt) {
    long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e < nE) atomicAdd(&cnt[color[e]], 1);
}
__global__ void k_color_fill(const int *__restrict__ color, long long nE, const int *__restrict__ off,
                             int *__restrict__ fill, int *__restrict__ list) {
    long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= nE) return;
    const int c = color[e];
    list[off[c] + atomicAdd(&fill[c], 1)] = (int)e;
}

// ---------------------------------------------------------------- close pairs (singular kernel)
// Close slots of element a: [a itself] followed by its dual-graph neighbours, at cbase[a] =
// xadj[a] + a. The Duffy blocks of each (a, partner) are computed once into closebuf.
__global__ void k_close_pairs(const long long *__restrict__ xadj, const int *__restrict__ adj,
                              const int *__restrict__ labT, const int *__restrict__ eprob,
                              const ProbParams *__restrict__ probs, long long nE,
                              int *__restrict__ cA, int *__restrict__ cB) {
    long long a = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= nE) return;
    const long long base = xadj[a] + a;
    const ProbParams &P = probs[eprob[a]];
    const bool use = labT[a] != 0 && duffy_close(P);
    cA[base] = use ? (int)a : -1;
    cB[base] = (int)a;
    for (long long j = xadj[a]; j < xadj[a + 1]; j++) {
        const int b = adj[j];
        cA[base + 1 + (j - xadj[a])] = (use && labT[b] != 0) ? (int)a : -1;
        cB[base + 1 + (j - xadj[a])] = b;
    }
}

__device__ __forceinline__ long long close_slot(const long long *__restrict__ xadj,
                                                const int *__restrict__ adj, int a, int b) {
    const long long base = xadj[a] + a;
    if (a == b) return base;
    long long lo = xadj[a], hi = xadj[a + 1] - 1;
    while (lo <= hi) {
        long long mid = (lo + hi) >> 1;
        int c = adj[mid];
        if (c == b) return base + 1 + (mid - xadj[a]);
        if (c < b) lo = mid + 1; else hi = mid - 1;
    }
    return -1;
}

// ---------------------------------------------------------------- pass arguments
struct PassArgs {
    const int *list;            // elements of this color
    int count;
    const int *T32, *labV, *eprob, *labT;
    const int *Tv;              // vertex table of the close-pair test (T32, except under DG: T32 then
                                // holds the element DOFs, which no two elements share)
    const double *EC, *adet;
    const float *EChi, *EClo;   // double-float split of EC
    const float *BCf;           // barycenters, double-float (BC_STRIDE floats per element)
    const float *adetf;         // |det| in FP32
    const ProbParams *probs;
    const long long *out_ptr, *in_ptr;
    const int *out_cnt;         // out-pair counts when the out-lists are the search's pool segments
                                // (out_ptr = segment starts, pB = the pool); null: out_ptr[T + 1] ends
    const int *pB, *inA;
    const long long *rowptr;
    const int *cols;
    double *vals;
    const long long *xadj;      // close-pair slots (singular kernels)
    const int *adj;
    const double *closebuf;     // (slots, 4, 3, 3)
    int *err;                   // [3] slot missing
    unsigned long long *n_subtri, *n_amb;
    unsigned long long *n_close;   // pairs integrated with the close-pair rule (from closebuf)
    unsigned long long *n_in, *n_cut;   // one-sided passes: (pair, outer point) items by class
    unsigned char *touched;     // mixed precision: slots that received a contribution
    const long long *zptr, *zidx;   // domain decomposition: element -> subdomain indicator (CSR)
};

constexpr int PASS_THREADS = 128;
constexpr int PASS_WARPS = PASS_THREADS / 32;
constexpr int ROWCACHE = 1536;   // columns of one row kept in shared memory

struct RowView {
    const int *c;   // column indices (shared or global)
    int n;
    long long base; // CSR slot of c[0]
};

__device__ __forceinline__ long long rv_find(const RowView &r, int col) {
    int lo = 0, hi = r.n - 1;
    while (lo <= hi) {
        int mid = (lo + hi) >> 1;
        int c = r.c[mid];
        if (c == col) return r.base + mid;
        if (c < col) lo = mid + 1; else hi = mid - 1;
    }
    return -1;
}

// Deterministic warp scatter of one column per lane (col < 0: nothing) with a vector over the
// warp's rows. Same-column lanes are summed in ascending lane order; the first lane of each group
// adds the sum to the CSR slots of the kept rows.
template <int NR>
__device__ __forceinline__ void warp_scatter(int col, const double *v, const RowView *rows,
                                             const bool *keep, double *vals, int *err,
                                             unsigned char *touched = nullptr) {
    const int lane = threadIdx.x & 31;
    const unsigned grp = __match_any_sync(FULL, col);
    const int gsize = __popc(grp);
    const bool leader = (__ffs(grp) - 1) == lane;
    const int maxn = __reduce_max_sync(FULL, (unsigned)gsize);
    double s[NR];
#pragma unroll
    for (int r = 0; r < NR; r++) s[r] = 0.0;
    unsigned m = grp;
    for (int it = 0; it < maxn; it++) {
        const int src = m ? __ffs(m) - 1 : lane;
        if (m) m &= m - 1;
#pragma unroll
        for (int r = 0; r < NR; r++) {
            const double t = __shfl_sync(FULL, v[r], src);
            if (it < gsize) s[r] += t;
        }
    }
    if (leader && col >= 0) {
#pragma unroll
        for (int r = 0; r < NR; r++) {
            if (!keep[r]) continue;
            const long long slot = rv_find(rows[r], col);
            if (slot < 0) { atomicOr(err, 1); continue; }
            vals[slot] += s[r];
            if (touched) touched[slot] = 1;
        }
    }
}

// Double-float variant (mixed precision): contributions and CSR values are DF pairs.
template <int NR>
__device__ __forceinline__ void warp_scatter_df(int col, const DF *v, const RowView *rows,
                                                const bool *keep, DF *vals, int *err,
                                                unsigned char *touched) {
    const int lane = threadIdx.x & 31;
    const unsigned grp = __match_any_sync(FULL, col);
    const int gsize = __popc(grp);
    const bool leader = (__ffs(grp) - 1) == lane;
    const int maxn = __reduce_max_sync(FULL, (unsigned)gsize);
    DF s[NR];
#pragma unroll
    for (int r = 0; r < NR; r++) s[r] = df_zero();
    unsigned m = grp;
    for (int it = 0; it < maxn; it++) {
        const int src = m ? __ffs(m) - 1 : lane;
        if (m) m &= m - 1;
#pragma unroll
        for (int r = 0; r < NR; r++) {
            DF t;
            t.hi = __shfl_sync(FULL, v[r].hi, src);
            t.lo = __shfl_sync(FULL, v[r].lo, src);
            if (it < gsize) s[r] = df_add(s[r], t);
        }
    }
    if (leader && col >= 0) {
#pragma unroll
        for (int r = 0; r < NR; r++) {
            if (!keep[r]) continue;
            const long long slot = rv_find(rows[r], col);
            if (slot < 0) { atomicOr(err, 1); continue; }
            vals[slot] = df_add(vals[slot], s[r]);
            if (touched) touched[slot] = 1;
        }
    }
}

__device__ __forceinline__ DF warp_sum_df(DF v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        DF t;
        t.hi = __shfl_xor_sync(FULL, v.hi, o);
        t.lo = __shfl_xor_sync(FULL, v.lo, o);
        // fixed pairing: the lower lane's value first, so both lanes compute the same sum
        const bool low = ((threadIdx.x & 31) & o) == 0;
        v = low ? df_add(v, t) : df_add(t, v);
    }
    return v;
}

// ---------------------------------------------------------------- rule-derived constants
template <typename R>
struct PassRuleT {
    R cx[MAXQ * 4];     // dx_k * psi_a(P_k)
    R cxx[MAXQ * 10];   // dx_k * psi_a psi_b (P_k), upper triangle
    R cyy[MAXQ * 10];   // dy_i * psi_a psi_b (P_i), upper triangle
    R cy[MAXQ * 4];     // dy_i * psi_a (P_i)
    R dxf[MAXQ];
    R pyf[MAXQ * 3];    // inner points P_i (FP32, any dimension)
    // Constant kernels: the inner rule's sums over a whole element, sum_i dy_i * (1, psi_a,
    // psi_a psi_b (upper triangle)), and (2D) its moments sum_i dy_i * (1, px, py, px^2, px py,
    // py^2) over the reference triangle.
    R insum[1 + 4 + 10];
    R mom[6];
    // sums over the outer points of cxx (upper triangle), cx and dxf, in that order: an outer
    // element's folds when every outer point's ball contains the partner (constant kernels)
    R xsum[10 + 4 + 1];
};
typedef PassRuleT<float> PassRule;


// ---------------------------------------------------------------- FP32 pair quadrature (2D)
// Inner quadrature of one outer point against triangle Q (relative to the outer point): returns
// the polygon point count and fills R (FP32, relative), with the certified FP32 geometry and the
// exact FP64 fallback.
__device__ __forceinline__ int cut_polygon(const F2 *Q, float sqf, const ProbParams &P,
                                           const double *x64, const double *E64, F2 *R,
                                           unsigned &namb) {
    bool amb = false;
    int n = fretriangulate(Q, sqf, P.caps, R, amb);
    if (amb) {
        namb++;
        double R64[18];
        n = xretriangulate(x64, E64, P.sqdelta, P.caps, R64);
        for (int j = 0; j < n; j++) R[j] = f2((float)(R64[2 * j] - x64[0]), (float)(R64[2 * j + 1] - x64[1]));
    }
    return n;
}

// Out side of pair (T, bT), retriangulate, mixed: L (sym, 6) and N (3x3) without the |T| factor.
__device__ void out_retri_mix(const ProbParams &P, const Rule &rule, const PassRule &pr,
                              const F2 *xs, const double *xs64, const float *pb, float rTb,
                              const double *Eb64, float *L, float *N, unsigned &nsub, unsigned &namb) {
    const F2 p0 = f2(pb[0], pb[1]), p1 = f2(pb[2], pb[3]), p2 = f2(pb[4], pb[5]);
    const F2 e1 = p1 - p0, e2 = p2 - p0;
    const float idet = 1.f / (e1.x * e2.y - e1.y * e2.x);
    const float sqf = P.sqdelta_f;
    for (int k = 0; k < rule.nPx; k++) {
        const F2 x = xs[k];
        const F2 Q[3] = {p0 - x, p1 - x, p2 - x};
        const int cls = fclassify(Q, sqf);
        if (cls == CLS_OUT) continue;
        float iL = 0.f, iN0 = 0.f, iN1 = 0.f, iN2 = 0.f;
        if (cls == CLS_IN) {
            nsub++;
            for (int i = 0; i < rule.nPy; i++) {
                const float px = rule.Pyf[2 * i], py = rule.Pyf[2 * i + 1];
                const float yx = Q[0].x + e1.x * px + e2.x * py;
                const float yy = Q[0].y + e1.y * px + e2.y * py;
                const float kw = kernel_f32(P, -yx, -yy) * rTb;
                iL = fmaf(kw, rule.dyf[i], iL);
                iN0 = fmaf(kw, pr.cy[3 * i + 0], iN0);
                iN1 = fmaf(kw, pr.cy[3 * i + 1], iN1);
                iN2 = fmaf(kw, pr.cy[3 * i + 2], iN2);
            }
        } else {
            F2 R[9];
            const int n = cut_polygon(Q, sqf, P, &xs64[2 * k], Eb64, R, namb);
            for (int r = 0; r + 2 < n; r++) {
                nsub++;
                const F2 A = R[0], B = R[r + 1] - R[0], C = R[r + 2] - R[0];
                const float rT = fabsf(B.x * C.y - B.y * C.x);
                for (int i = 0; i < rule.nPy; i++) {
                    const float px = rule.Pyf[2 * i], py = rule.Pyf[2 * i + 1];
                    const float yx = A.x + B.x * px + C.x * py;
                    const float yy = A.y + B.y * px + C.y * py;
                    const float kw = kernel_f32(P, -yx, -yy) * rT * rule.dyf[i];
                    const float dxr = yx - Q[0].x, dyr = yy - Q[0].y;
                    const float r0 = (e2.y * dxr - e2.x * dyr) * idet;
                    const float r1 = (e1.x * dyr - e1.y * dxr) * idet;
                    iL += kw;
                    iN0 = fmaf(kw, 1.f - r0 - r1, iN0);
                    iN1 = fmaf(kw, r0, iN1);
                    iN2 = fmaf(kw, r1, iN2);
                }
            }
        }
#pragma unroll
        for (int ab = 0; ab < 6; ab++) L[ab] = fmaf(pr.cxx[6 * k + ab], iL, L[ab]);
#pragma unroll
        for (int a = 0; a < 3; a++) {
            const float c = pr.cx[3 * k + a];
            N[3 * a + 0] = fmaf(c, iN0, N[3 * a + 0]);
            N[3 * a + 1] = fmaf(c, iN1, N[3 * a + 1]);
            N[3 * a + 2] = fmaf(c, iN2, N[3 * a + 2]);
        }
    }
}

// In side of pair (aT, T), retriangulate, mixed: LP (sym, 6, T's vertices) and NP[a][b]
// (a: aT's vertex, b: T's vertex) without the |aT| factor.
__device__ void in_retri_mix(const ProbParams &P, const Rule &rule, const PassRule &pr,
                             const float *pa, const double *Ea64, const F2 *tl, const F2 *yT,
                             float rTT, float idetT, const double *ET64, float *LP, float *NP,
                             unsigned &nsub, unsigned &namb) {
    const F2 a0 = f2(pa[0], pa[1]), ea1 = f2(pa[2] - pa[0], pa[3] - pa[1]), ea2 = f2(pa[4] - pa[0], pa[5] - pa[1]);
    const F2 e1 = tl[1] - tl[0], e2 = tl[2] - tl[0];
    const float sqf = P.sqdelta_f;
    for (int k = 0; k < rule.nPx; k++) {
        const float px = rule.Pxf[2 * k], py = rule.Pxf[2 * k + 1];
        const F2 x = f2(a0.x + ea1.x * px + ea2.x * py, a0.y + ea1.y * px + ea2.y * py);
        const F2 Q[3] = {tl[0] - x, tl[1] - x, tl[2] - x};
        const int cls = fclassify(Q, sqf);
        if (cls == CLS_OUT) continue;
        float i0 = 0.f, i1 = 0.f, i2 = 0.f;
        float lp[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
        if (cls == CLS_IN) {
            for (int i = 0; i < rule.nPy; i++) {
                const F2 y = yT[i] - x;
                const float kw = kernel_f32(P, -y.x, -y.y) * rTT;
                i0 = fmaf(kw, pr.cy[3 * i + 0], i0);
                i1 = fmaf(kw, pr.cy[3 * i + 1], i1);
                i2 = fmaf(kw, pr.cy[3 * i + 2], i2);
#pragma unroll
                for (int ab = 0; ab < 6; ab++) lp[ab] = fmaf(kw, pr.cyy[6 * i + ab], lp[ab]);
            }
        } else {
            double x64[2];
            xtoPhys<2>(Ea64, &rule.Px[2 * k], x64);
            F2 R[9];
            const int n = cut_polygon(Q, sqf, P, x64, ET64, R, namb);
            for (int r = 0; r + 2 < n; r++) {
                const F2 A = R[0], B = R[r + 1] - R[0], C = R[r + 2] - R[0];
                const float rT = fabsf(B.x * C.y - B.y * C.x);
                for (int i = 0; i < rule.nPy; i++) {
                    const float qx = rule.Pyf[2 * i], qy = rule.Pyf[2 * i + 1];
                    const float yx = A.x + B.x * qx + C.x * qy;
                    const float yy = A.y + B.y * qx + C.y * qy;
                    const float kw = kernel_f32(P, -yx, -yy) * rT * rule.dyf[i];
                    const float dxr = yx - Q[0].x, dyr = yy - Q[0].y;
                    const float r0 = (e2.y * dxr - e2.x * dyr) * idetT;
                    const float r1 = (e1.x * dyr - e1.y * dxr) * idetT;
                    const float s[3] = {1.f - r0 - r1, r0, r1};
                    i0 = fmaf(kw, s[0], i0);
                    i1 = fmaf(kw, s[1], i1);
                    i2 = fmaf(kw, s[2], i2);
                    lp[0] = fmaf(kw, s[0] * s[0], lp[0]); lp[1] = fmaf(kw, s[0] * s[1], lp[1]);
                    lp[2] = fmaf(kw, s[0] * s[2], lp[2]); lp[3] = fmaf(kw, s[1] * s[1], lp[3]);
                    lp[4] = fmaf(kw, s[1] * s[2], lp[4]); lp[5] = fmaf(kw, s[2] * s[2], lp[5]);
                }
            }
        }
        const float dk = pr.dxf[k];
#pragma unroll
        for (int ab = 0; ab < 6; ab++) LP[ab] = fmaf(dk, lp[ab], LP[ab]);
#pragma unroll
        for (int a = 0; a < 3; a++) {
            const float c = pr.cx[3 * k + a];
            NP[3 * a + 0] = fmaf(c, i0, NP[3 * a + 0]);
            NP[3 * a + 1] = fmaf(c, i1, NP[3 * a + 1]);
            NP[3 * a + 2] = fmaf(c, i2, NP[3 * a + 2]);
        }
    }
}

// ---------------------------------------------------------------- FP64 pair quadrature (2D)
// Reference arithmetic (integration.cpp:345-540) split by side.
__device__ void out_retri_f64(const ProbParams &P, const Rule &rule, const double *xs64,
                              const double *Eb, int la, int lb, double *L, double *N, unsigned &nsub, int *err) {
    double R[18];
    for (int k = 0; k < rule.nPx; k++) {
        const double *x = &xs64[2 * k];
        const int Rdx = xretriangulate(x, Eb, P.sqdelta, P.caps, R);
        double iL = 0, iN[3] = {0, 0, 0};
        for (int r = 0; r + 2 < Rdx; r++) {
            nsub++;
            const double tri[6] = {R[0], R[1], R[2 * r + 2], R[2 * r + 3], R[2 * r + 4], R[2 * r + 5]};
            const double rTdet = xabsDet2(tri);
            for (int i = 0; i < rule.nPy; i++) {
                double y[2];
                y[0] = (tri[2] - tri[0]) * rule.Py[2 * i] + (tri[4] - tri[0]) * rule.Py[2 * i + 1] + tri[0];
                y[1] = (tri[3] - tri[1]) * rule.Py[2 * i] + (tri[5] - tri[1]) * rule.Py[2 * i + 1] + tri[1];
                const double w = kernel_f64<2>(P, x, la, y, lb, err) * rule.dy[i] * rTdet;
                iL += w;
                double ref[2];
                if (!xtoRef(Eb, y, ref)) atomicOr(&err[4], 1);
                iN[0] += (1.0 - ref[0] - ref[1]) * w;
                iN[1] += ref[0] * w;
                iN[2] += ref[1] * w;
            }
        }
        for (int a = 0; a < 3; a++) {
            const double pa = rule.psix[3 * k + a] * rule.dx[k];
            for (int b = a; b < 3; b++) L[sym_idx<3>(a, b)] += pa * rule.psix[3 * k + b] * iL;
            for (int b = 0; b < 3; b++) N[3 * a + b] += pa * iN[b];
        }
    }
}

__device__ void in_retri_f64(const ProbParams &P, const Rule &rule, const double *Ea,
                             const double *ET, int la, int lT, double *LP, double *NP, unsigned &nsub, int *err) {
    double R[18];
    for (int k = 0; k < rule.nPx; k++) {
        double x[2];
        xtoPhys<2>(Ea, &rule.Px[2 * k], x);
        const int Rdx = xretriangulate(x, ET, P.sqdelta, P.caps, R);
        double iNP[3] = {0, 0, 0};
        for (int r = 0; r + 2 < Rdx; r++) {
            const double tri[6] = {R[0], R[1], R[2 * r + 2], R[2 * r + 3], R[2 * r + 4], R[2 * r + 5]};
            const double rTdet = xabsDet2(tri);
            for (int i = 0; i < rule.nPy; i++) {
                double y[2];
                y[0] = (tri[2] - tri[0]) * rule.Py[2 * i] + (tri[4] - tri[0]) * rule.Py[2 * i + 1] + tri[0];
                y[1] = (tri[3] - tri[1]) * rule.Py[2 * i] + (tri[5] - tri[1]) * rule.Py[2 * i + 1] + tri[1];
                const double w = kernel_f64<2>(P, y, lT, x, la, err) * rule.dy[i] * rTdet;
                double ref[2];
                if (!xtoRef(ET, y, ref)) atomicOr(&err[4], 1);
                const double s[3] = {1.0 - ref[0] - ref[1], ref[0], ref[1]};
                for (int b = 0; b < 3; b++) iNP[b] += s[b] * w;
                const double wl = w * rule.dx[k];
                for (int a = 0; a < 3; a++)
                    for (int b = a; b < 3; b++) LP[sym_idx<3>(a, b)] += s[a] * s[b] * wl;
            }
        }
        for (int a = 0; a < 3; a++) {
            const double pa = rule.psix[3 * k + a] * rule.dx[k];
            for (int b = 0; b < 3; b++) NP[3 * a + b] += pa * iNP[b];
        }
    }
}

// ---------------------------------------------------------------- barycenter (2D / 3D)
// integrate_baryCenter (integration.cpp:910-1018): out side only (the prime blocks are zero).
template <int DIM, int PREC>
__device__ void out_bary(const ProbParams &P, const Rule &rule, const PassRule &pr, const float *xsf,
                         const double *xs64, const float *pb, const double *Eb64, double adetb,
                         int la, int lb, double *L, double *N, unsigned &nsub, unsigned &namb, int *err) {
    constexpr int dV = DIM + 1;
    constexpr int NS = dV * (dV + 1) / 2;
    double b64[DIM];
    xbary<DIM>(Eb64, b64);
    float bf[DIM];
#pragma unroll
    for (int j = 0; j < DIM; j++) {
        float s = pb[j];
#pragma unroll
        for (int i = 1; i <= DIM; i++) s += pb[DIM * i + j];
        bf[j] = s / (float)dV;
    }
    const float sqlo = P.sqdelta_f * (1.f - MARG_D), sqhi = P.sqdelta_f * (1.f + MARG_D);
    for (int k = 0; k < rule.nPx; k++) {
        bool inside;
        if (PREC == PREC_F64) {
            inside = xbaryInside<DIM>(&xs64[DIM * k], b64, P.sqdelta);
        } else {
            float d2 = 0.f;
#pragma unroll
            for (int j = 0; j < DIM; j++) { float d = xsf[DIM * k + j] - bf[j]; d2 = fmaf(d, d, d2); }
            if (d2 < sqlo) inside = true;
            else if (d2 > sqhi) inside = false;
            else { namb++; inside = xbaryInside<DIM>(&xs64[DIM * k], b64, P.sqdelta); }
        }
        if (!inside) continue;
        nsub++;
        if (PREC == PREC_F64) {
            double iL = 0, iN[dV];
#pragma unroll
            for (int j = 0; j < dV; j++) iN[j] = 0;
            for (int i = 0; i < rule.nPy; i++) {
                double y[DIM];
                xtoPhys<DIM>(Eb64, &rule.Py[DIM * i], y);
                const double ker = kernel_f64<DIM>(P, &xs64[DIM * k], la, y, lb, err);
                iL += adetb * ker * rule.dy[i];
                const double kerP = kernel_f64<DIM>(P, y, lb, &xs64[DIM * k], la, err);
#pragma unroll
                for (int j = 0; j < dV; j++) iN[j] += rule.psiy[dV * i + j] * kerP * rule.dy[i] * adetb;
            }
            for (int a = 0; a < dV; a++) {
                const double pa = 2.0 * rule.psix[dV * k + a] * rule.dx[k];
                for (int j = a; j < dV; j++) L[sym_idx<dV>(a, j)] += pa * rule.psix[dV * k + j] * iL;
                for (int j = 0; j < dV; j++) N[dV * a + j] += pa * iN[j];
            }
        } else {
            float iL = 0.f, iN[dV];
#pragma unroll
            for (int j = 0; j < dV; j++) iN[j] = 0.f;
            for (int i = 0; i < rule.nPy; i++) {
                float y[DIM];
#pragma unroll
                for (int j = 0; j < DIM; j++) {
                    float s = pb[j];
#pragma unroll
                    for (int c = 0; c < DIM; c++) s = fmaf(pb[DIM * (c + 1) + j] - pb[j], (float)rule.Py[DIM * i + c], s);
                    y[j] = s;
                }
                float kw;
                if (DIM == 2) kw = kernel_f32(P, xsf[2 * k] - y[0], xsf[2 * k + 1] - y[1]);
                else kw = P.kc_f;
                iL = fmaf(kw, rule.dyf[i], iL);
#pragma unroll
                for (int j = 0; j < dV; j++) iN[j] = fmaf(kw, pr.cy[dV * i + j], iN[j]);
            }
            const float rb = (float)adetb;
            for (int a = 0; a < dV; a++) {
                const double pa = 2.0 * (double)pr.cx[dV * k + a];
                for (int j = a; j < dV; j++) L[sym_idx<dV>(a, j)] += (double)(pr.cxx[NS * k + sym_idx<dV>(a, j)] * 2.f * iL * rb);
                for (int j = 0; j < dV; j++) N[dV * a + j] += pa * (double)(iN[j] * rb);
            }
        }
    }
}

// ---------------------------------------------------------------- the pass kernel
// Domain-decomposition weight of the pair (A, B) (Cassemble.cpp:649-657): 1 / the number of
// subdomains both elements belong to (evaluateZeta, mathhelpers.cpp:19-38: the intersection of
// their sorted indicator rows).
__device__ __forceinline__ double zeta_weight(const long long *__restrict__ zptr, const long long *__restrict__ zidx,
                                              long long A, long long B) {
    long long i = zptr[A], ie = zptr[A + 1], j = zptr[B], je = zptr[B + 1];
    long long n = 0;
    while (i < ie && j < je) {
        const long long x = zidx[i], y = zidx[j];
        if (x < y) i++;
        else if (y < x) j++;
        else { n++; i++; j++; }
    }
    return 1.0 / (double)n;
}

template <int DIM, int PREC>
__global__ void __launch_bounds__(PASS_THREADS) k_pass(PassArgs a, Rule rule, PassRule pr) {
    constexpr int dV = DIM + 1;
    constexpr int NS = dV * (dV + 1) / 2;
    __shared__ double s_x64[PASS_WARPS][MAXQ * DIM];
    __shared__ float s_xf[PASS_WARPS][MAXQ * DIM];
    __shared__ F2 s_yT[PASS_WARPS][MAXQ];
    extern __shared__ int s_dyn[];   // PASS_WARPS * dV * ROWCACHE column indices
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    int *s_cols = s_dyn + wib * dV * ROWCACHE;
    const long long gw = (long long)blockIdx.x * PASS_WARPS + wib;
    const long long nw = (long long)gridDim.x * PASS_WARPS;
    unsigned nsub = 0, namb = 0, nclose = 0;
    for (long long idx = gw; idx < a.count; idx += nw) {
        const int T = a.list[idx];
        int tv[dV];
        bool keep[dV];
        bool any = false;
#pragma unroll
        for (int r = 0; r < dV; r++) {
            tv[r] = a.T32[(long long)T * dV + r];
            keep[r] = a.labV[tv[r]] > 0;
            any |= keep[r];
        }
        if (!any || a.labT[T] == 0) continue;
        // an element without any pair (a ball smaller than the element can stay strictly inside
        // it, which the retriangulation counts as no polygon) adds nothing, and its row pattern
        // holds none of its columns
        if (a.out_ptr[T] == a.out_ptr[T + 1] && (!a.in_ptr || a.in_ptr[T] == a.in_ptr[T + 1])) continue;
        const ProbParams P = a.probs[a.eprob[T]];
        // rows of T's vertices: column lists in shared memory when they fit
        RowView rows[dV];
#pragma unroll
        for (int r = 0; r < dV; r++) {
            const long long b = a.rowptr[tv[r]];
            const int n = (int)(a.rowptr[tv[r] + 1] - b);
            rows[r].n = n;
            rows[r].base = b;
            if (n <= ROWCACHE) {
                for (int i = lane; i < n; i += 32) s_cols[r * ROWCACHE + i] = a.cols[b + i];
                rows[r].c = s_cols + r * ROWCACHE;
            } else {
                rows[r].c = a.cols + b;
            }
        }
        const double *ET64 = &a.EC[(long long)T * DIM * dV];
        float ohi[DIM], olo[DIM];
#pragma unroll
        for (int j = 0; j < DIM; j++) { ohi[j] = a.EChi[(long long)T * DIM * dV + j]; olo[j] = a.EClo[(long long)T * DIM * dV + j]; }
        float tl[DIM * dV];
#pragma unroll
        for (int j = 0; j < DIM * dV; j++)
            tl[j] = (a.EChi[(long long)T * DIM * dV + j] - ohi[j % DIM]) + (a.EClo[(long long)T * DIM * dV + j] - olo[j % DIM]);
        const double adetT = a.adet[T];
        for (int k = lane; k < rule.nPx; k += 32) {
            xtoPhys<DIM>(ET64, &rule.Px[DIM * k], &s_x64[wib][DIM * k]);
#pragma unroll
            for (int j = 0; j < DIM; j++) s_xf[wib][DIM * k + j] = (float)(s_x64[wib][DIM * k + j] - ET64[j]);
        }
        if (DIM == 2) {
            const F2 e1 = f2(tl[2] - tl[0], tl[3] - tl[1]), e2 = f2(tl[4] - tl[0], tl[5] - tl[1]);
            for (int i = lane; i < rule.nPy; i += 32) {
                const float px = rule.Pyf[2 * i], py = rule.Pyf[2 * i + 1];
                s_yT[wib][i] = f2(tl[0] + e1.x * px + e2.x * py, tl[1] + e1.y * px + e2.y * py);
            }
        }
        __syncwarp();
        double D[NS];   // diagonal block A[T, T] (upper triangle): termLocal + termLocalPrime
#pragma unroll
        for (int i = 0; i < NS; i++) D[i] = 0.0;
        const bool frac_close = duffy_close(P);   // fractional or weakSingular close blocks
        // ---------------- out side: pairs (T, bT)
        const long long ob = a.out_ptr[T], oe = a.out_ptr[T + 1];
        for (long long p0 = ob; p0 < oe; p0 += 32) {
            const long long p = p0 + lane;
            const bool act = p < oe;
            const int bT = act ? a.pB[p] : T;
            int bv[dV];
#pragma unroll
            for (int r = 0; r < dV; r++) bv[r] = a.T32[(long long)bT * dV + r];
            double Nd[dV * dV], Dp[NS];   // the pair's termNonloc and termLocal (upper triangle)
#pragma unroll
            for (int i = 0; i < dV * dV; i++) Nd[i] = 0.0;
#pragma unroll
            for (int i = 0; i < NS; i++) Dp[i] = 0.0;
            if (act) {
                const double *Eb64 = &a.EC[(long long)bT * DIM * dV];
                bool done = false;
                if (DIM == 2 && frac_close) {
                    bool close = (bT == T);
                    if (a.Tv == a.T32) {
                        for (int i = 0; i < dV; i++)
                            for (int j = 0; j < dV; j++) close |= (tv[i] == bv[j]);
                    } else {
                        for (int i = 0; i < dV; i++)
                            for (int j = 0; j < dV; j++) close |= (a.Tv[(long long)T * dV + i] == a.Tv[(long long)bT * dV + j]);
                    }
                    if (close) {
                        nclose++;
                        const long long cs = close_slot(a.xadj, a.adj, T, bT);
                        if (cs < 0) { atomicOr(&a.err[3], 1); }
                        else {
                            const double *cb = &a.closebuf[cs * 36];
                            for (int i = 0; i < 3; i++)
                                for (int j = i; j < 3; j++) Dp[sym_idx<dV>(i, j)] += cb[3 * i + j];
                            for (int i = 0; i < 9; i++) Nd[i] = cb[9 + i];
                        }
                        done = true;
                    }
                }
                if (!done) {
                    if (P.remote == MTH_BARYCENTER) {
                        float pb[DIM * dV];
#pragma unroll
                        for (int j = 0; j < DIM * dV; j++)
                            pb[j] = (a.EChi[(long long)bT * DIM * dV + j] - ohi[j % DIM]) + (a.EClo[(long long)bT * DIM * dV + j] - olo[j % DIM]);
                        double Ls[NS];
#pragma unroll
                        for (int i = 0; i < NS; i++) Ls[i] = 0.0;
                        out_bary<DIM, PREC>(P, rule, pr, s_xf[wib], s_x64[wib], pb, Eb64, a.adet[bT], a.labT[T], a.labT[bT], Ls, Nd, nsub, namb, a.err);
#pragma unroll
                        for (int i = 0; i < NS; i++) Dp[i] += Ls[i] * adetT;
#pragma unroll
                        for (int i = 0; i < dV * dV; i++) Nd[i] *= adetT;
                    } else if (DIM == 2 && PREC == PREC_F64 && P.remote != MTH_RETRIANGULATE) {
                        double Ls[6] = {0, 0, 0, 0, 0, 0};
                        rule_out_f64(P, P.remote, rule, ET64, Eb64, a.adet[bT], a.labT[T], a.labT[bT], Ls, Nd, nsub, a.err);
                        const double sT = P.remote == MTH_BARY_RT ? 1.0 : adetT;   // baryCenterRT carries its factor
                        for (int i = 0; i < 6; i++) Dp[i] += Ls[i] * sT;
                        for (int i = 0; i < 9; i++) Nd[i] *= sT;
                    } else if (DIM == 2) {
                        if (PREC == PREC_F64) {
                            double Ls[6] = {0, 0, 0, 0, 0, 0};
                            out_retri_f64(P, rule, s_x64[wib], Eb64, a.labT[T], a.labT[bT], Ls, Nd, nsub, a.err);
                            for (int i = 0; i < 6; i++) Dp[i] += Ls[i] * adetT;
                            for (int i = 0; i < 9; i++) Nd[i] *= adetT;
                        } else {
                            float pb[6];
#pragma unroll
                            for (int j = 0; j < 6; j++)
                                pb[j] = (a.EChi[(long long)bT * 6 + j] - ohi[j & 1]) + (a.EClo[(long long)bT * 6 + j] - olo[j & 1]);
                            float Lf[6] = {0, 0, 0, 0, 0, 0}, Nf[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
                            out_retri_mix(P, rule, pr, (const F2 *)s_xf[wib], s_x64[wib], pb, (float)a.adet[bT], Eb64, Lf, Nf, nsub, namb);
                            for (int i = 0; i < 6; i++) Dp[i] += (double)Lf[i] * adetT;
                            for (int i = 0; i < 9; i++) Nd[i] = (double)Nf[i] * adetT;
                        }
                    }
                }
            }
            {   // the pair's weight (1 without domain decomposition)
                const double w = (act && P.zeta) ? zeta_weight(a.zptr, a.zidx, T, bT) : 1.0;
#pragma unroll
                for (int i = 0; i < NS; i++) D[i] += Dp[i] * w;
#pragma unroll
                for (int i = 0; i < dV * dV; i++) Nd[i] *= w;
            }
            // termNonloc -> A[T[a], bT[b]] with the minus sign (Cassemble.cpp:744-749)
#pragma unroll
            for (int b = 0; b < dV; b++) {
                if (PREC == PREC_MIX) {
                    DF v[dV];
#pragma unroll
                    for (int r = 0; r < dV; r++) v[r] = df_from_double(-Nd[dV * r + b]);
                    warp_scatter_df<dV>(act ? bv[b] : -1, v, rows, keep, (DF *)a.vals, &a.err[3], a.touched);
                } else {
                    double v[dV];
#pragma unroll
                    for (int r = 0; r < dV; r++) v[r] = -Nd[dV * r + b];
                    warp_scatter<dV>(act ? bv[b] : -1, v, rows, keep, a.vals, &a.err[3], a.touched);
                }
            }
            __syncwarp();
        }
        // ---------------- in side: pairs (aT, T) (prime blocks; zero for the barycenter rule)
        const bool prime = (DIM == 2) && (P.remote == MTH_RETRIANGULATE || P.remote == MTH_NOTRUNC || frac_close);
        if (prime) {
            const long long ib = a.in_ptr[T], ie = a.in_ptr[T + 1];
            const F2 tlf[3] = {f2(tl[0], tl[1]), f2(tl[2], tl[3]), f2(tl[4], tl[5])};
            const float idetT = 1.f / ((tl[2] - tl[0]) * (tl[5] - tl[1]) - (tl[3] - tl[1]) * (tl[4] - tl[0]));
            for (long long q0 = ib; q0 < ie; q0 += 32) {
                const long long q = q0 + lane;
                const bool act = q < ie;
                const int aT = act ? a.inA[q] : T;
                int av[3];
#pragma unroll
                for (int r = 0; r < 3; r++) av[r] = a.T32[(long long)aT * 3 + r];
                double NPd[9], Dp[6];   // the pair's termNonlocPrime and termLocalPrime (upper triangle)
#pragma unroll
                for (int i = 0; i < 9; i++) NPd[i] = 0.0;
#pragma unroll
                for (int i = 0; i < 6; i++) Dp[i] = 0.0;
                if (act) {
                    const double *Ea64 = &a.EC[(long long)aT * 6];
                    const double adetA = a.adet[aT];
                    bool done = false;
                    if (frac_close) {
                        bool close = (aT == T);
                        if (a.Tv == a.T32) {
                            for (int i = 0; i < 3; i++)
                                for (int j = 0; j < 3; j++) close |= (tv[i] == av[j]);
                        } else {
                            for (int i = 0; i < 3; i++)
                                for (int j = 0; j < 3; j++) close |= (a.Tv[(long long)T * 3 + i] == a.Tv[(long long)aT * 3 + j]);
                        }
                        if (close) {
                            const long long cs = close_slot(a.xadj, a.adj, aT, T);
                            if (cs < 0) { atomicOr(&a.err[3], 1); }
                            else {
                                const double *cb = &a.closebuf[cs * 36];
                                // LP[a][b] -> A[T[b], T[a]]: the diagonal block of T takes LP^T
                                for (int i = 0; i < 3; i++)
                                    for (int j = i; j < 3; j++) Dp[sym_idx<3>(i, j)] += cb[18 + 3 * j + i];
                                for (int i = 0; i < 9; i++) NPd[i] = cb[27 + i];
                            }
                            done = true;
                        }
                    }
                    if (!done && PREC == PREC_F64 && P.remote == MTH_NOTRUNC) {
                        double LP[6] = {0, 0, 0, 0, 0, 0};
                        rule_notrunc_prime(P, rule, Ea64, ET64, adetT, a.labT[aT], a.labT[T], LP, NPd, a.err);
                        for (int i = 0; i < 6; i++) Dp[i] += LP[i] * adetA;
                        for (int i = 0; i < 9; i++) NPd[i] *= adetA;
                    }
                    if (!done && P.remote == MTH_RETRIANGULATE) {
                        if (PREC == PREC_F64) {
                            double LP[6] = {0, 0, 0, 0, 0, 0};
                            in_retri_f64(P, rule, Ea64, ET64, a.labT[aT], a.labT[T], LP, NPd, nsub, a.err);
                            for (int i = 0; i < 6; i++) Dp[i] += LP[i] * adetA;
                            for (int i = 0; i < 9; i++) NPd[i] *= adetA;
                        } else {
                            float pa[6];
#pragma unroll
                            for (int j = 0; j < 6; j++)
                                pa[j] = (a.EChi[(long long)aT * 6 + j] - ohi[j & 1]) + (a.EClo[(long long)aT * 6 + j] - olo[j & 1]);
                            float LPf[6] = {0, 0, 0, 0, 0, 0}, NPf[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
                            in_retri_mix(P, rule, pr, pa, Ea64, tlf, s_yT[wib], (float)adetT, idetT, ET64, LPf, NPf, nsub, namb);
                            for (int i = 0; i < 6; i++) Dp[i] += (double)LPf[i] * adetA;
                            for (int i = 0; i < 9; i++) NPd[i] = (double)NPf[i] * adetA;
                        }
                    }
                }
                {   // the pair's weight (1 without domain decomposition)
                    const double w = (act && P.zeta) ? zeta_weight(a.zptr, a.zidx, aT, T) : 1.0;
#pragma unroll
                    for (int i = 0; i < 6; i++) D[i] += Dp[i] * w;
#pragma unroll
                    for (int i = 0; i < 9; i++) NPd[i] *= w;
                }
                // termNonlocPrime[a][b] -> A[T[b], aT[a]] with the minus sign (Cassemble.cpp:761-766)
#pragma unroll
                for (int c = 0; c < 3; c++) {
                    if (PREC == PREC_MIX) {
                        DF v[3];
#pragma unroll
                        for (int r = 0; r < 3; r++) v[r] = df_from_double(-NPd[3 * c + r]);
                        warp_scatter_df<3>(act ? av[c] : -1, v, rows, keep, (DF *)a.vals, &a.err[3], a.touched);
                    } else {
                        double v[3];
#pragma unroll
                        for (int r = 0; r < 3; r++) v[r] = -NPd[3 * c + r];
                        warp_scatter<3>(act ? av[c] : -1, v, rows, keep, a.vals, &a.err[3], a.touched);
                    }
                }
                __syncwarp();
            }
        }
        // ---------------- diagonal block: fixed-tree warp reduction, lane 0 adds
#pragma unroll
        for (int i = 0; i < NS; i++) D[i] = warp_sum(D[i]);
        if (lane == 0) {
            for (int r = 0; r < dV; r++) {
                if (!keep[r]) continue;
                for (int c = 0; c < dV; c++) {
                    const long long slot = rv_find(rows[r], tv[c]);
                    if (slot < 0) { atomicOr(&a.err[3], 1); continue; }
                    const double dv = D[r <= c ? sym_idx<dV>(r, c) : sym_idx<dV>(c, r)];
                    if (PREC == PREC_MIX) {
                        DF *vv = (DF *)a.vals;
                        vv[slot] = df_add(vv[slot], df_from_double(dv));
                    } else {
                        a.vals[slot] += dv;
                    }
                    if (a.touched) a.touched[slot] = 1;
                }
            }
        }
        __syncwarp();
    }
    nsub = warp_sum(nsub);
    namb = warp_sum(namb);
    nclose = warp_sum(nclose);
    if (lane == 0) {
        if (nsub && a.n_subtri) atomicAdd(a.n_subtri, (unsigned long long)nsub);
        if (namb && a.n_amb) atomicAdd(a.n_amb, (unsigned long long)namb);
        if (nclose && a.n_close) atomicAdd(a.n_close, (unsigned long long)nclose);
    }
}

}  // namespace nlg
