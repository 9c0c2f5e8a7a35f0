// GB300 (sm_103a) nonlocal stiffness-matrix / load-vector assembly.
//
// Pipeline of one assembly (all on the device, one stream):
//   prep      int64 mesh -> int32 connectivity, element coordinates, |det| (FP64)
//   dual      vertex->element incidence and vertex-sharing element adjacency (replaces
//             METIS_MeshToDual(ncommon=1), src/Cassemble.cpp:391-417)
//   bfs       one warp per outer element: breadth-first search over the dual graph with the
//             bit-exact interaction predicate (src/Cassemble.cpp:595-783); emits the ordered
//             interacting pairs (aT, bT)
//   pairs     compaction into aT-major pair arrays; transposed (bT-major) lists
//   pattern   CSR sparsity pattern: row u collects the vertices of every element touching an
//             element incident to u (src/Cassemble.cpp:721-770 index rules)
//   quad      per-pair quadrature of the four local blocks (src/integration.cpp) and their
//             scatter into CSR slots through 128-bit fixed-point atomics (order independent,
//             so run-to-run identical)
//   finish    fixed point -> FP64, exact zeros dropped (arma::sp_mat semantics)
#include "../../include/nlfem_gpu.h"
#include "geometry.cuh"
#include "primitives.cuh"
#include "quadrature.cuh"
#include "passes.cuh"
#include "passes_mix.cuh"
#include "passes_bary.cuh"
#include "passes_vec.cuh"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

namespace nlg {

// ======================================================================= device kernels
__device__ __forceinline__ int find_prob(const int *off, int n, long long e) {
    int lo = 0, hi = n - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if ((long long)off[mid] <= e) lo = mid; else hi = mid - 1;
    }
    return lo;
}

template <int DIM>
__global__ void k_prep_elements(const long long *__restrict__ T64, const long long *__restrict__ lab64,
                                const double *__restrict__ V, const int *__restrict__ eoff,
                                const int *__restrict__ voff, int nProb, long long nE,
                                int *__restrict__ T32, int *__restrict__ labT, int *__restrict__ eprob,
                                double *__restrict__ EC, double *__restrict__ adet,
                                float *__restrict__ EChi, float *__restrict__ EClo,
                                float *__restrict__ adetf, float *__restrict__ BCf) {
    constexpr int dV = DIM + 1;
    long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= nE) return;
    const int p = find_prob(eoff, nProb, e);
    const int vo = voff[p];
    double E[DIM * dV];
#pragma unroll
    for (int k = 0; k < dV; k++) {
        int v = (int)T64[e * dV + k] + vo;
        T32[e * dV + k] = v;
#pragma unroll
        for (int j = 0; j < DIM; j++) {
            E[DIM * k + j] = V[(long long)v * DIM + j];
            EC[e * DIM * dV + DIM * k + j] = E[DIM * k + j];
            const float hi = (float)E[DIM * k + j];
            EChi[e * DIM * dV + DIM * k + j] = hi;
            EClo[e * DIM * dV + DIM * k + j] = (float)(E[DIM * k + j] - (double)hi);
        }
    }
    {   // barycenter (mathhelpers.cpp:184-196), split like the vertex coordinates
        double b[DIM];
        xbary<DIM>(E, b);
        float *o = &BCf[e * BC_STRIDE<DIM>];
#pragma unroll
        for (int j = 0; j < DIM; j++) {
            const float hi = (float)b[j];
            o[j] = hi;
            o[BC_STRIDE<DIM> / 2 + j] = (float)(b[j] - (double)hi);
        }
        if (DIM == 3) { o[3] = 0.f; o[7] = 0.f; }
    }
    long long l = lab64[e];
    labT[e] = (int)(l > 2147483647LL ? 2147483647LL : (l < -2147483647LL ? -2147483647LL : l));
    eprob[e] = p;
    // absDet(E, dim) with the cofactor determinant (mathhelpers.cpp:112-129)
    double det;
    if (DIM == 2) {
        double a = xsub(E[2], E[0]), b = xsub(E[4], E[0]);
        double c = xsub(E[3], E[1]), d = xsub(E[5], E[1]);
        det = xsub(xmul(a, d), xmul(c, b));
    } else {
        double M[3][3];
        for (int i = 1; i < 4; i++)
            for (int j = 0; j < 3; j++) M[j][i - 1] = xsub(E[j + 3 * i], E[j]);
        double c0 = xsub(xmul(M[1][1], M[2][2]), xmul(M[1][2], M[2][1]));
        double c1 = xsub(xmul(M[1][0], M[2][2]), xmul(M[1][2], M[2][0]));
        double c2 = xsub(xmul(M[1][0], M[2][1]), xmul(M[1][1], M[2][0]));
        det = xadd(xsub(xmul(M[0][0], c0), xmul(M[0][1], c1)), xmul(M[0][2], c2));
    }
    adet[e] = fabs(det);
    adetf[e] = (float)fabs(det);
}

__global__ void k_prep_vertices(const long long *__restrict__ lab64, const int *__restrict__ voff,
                                int nProb, long long nV, int *__restrict__ labV, int *__restrict__ vprob) {
    long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= nV) return;
    long long l = lab64[v];
    labV[v] = (int)(l > 2147483647LL ? 2147483647LL : (l < -2147483647LL ? -2147483647LL : l));
    vprob[v] = find_prob(voff, nProb, v);
}

// ------------------------------------------------------------------ dual graph
__global__ void k_vinc_count(const int *__restrict__ T32, long long n, int *__restrict__ vcnt) {
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) atomicAdd(&vcnt[T32[i]], 1);
}
__global__ void k_vinc_fill(const int *__restrict__ T32, long long n, int dV,
                            const long long *__restrict__ vptr, int *__restrict__ vfill,
                            int *__restrict__ vel) {
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int v = T32[i];
    long long pos = vptr[v] + atomicAdd(&vfill[v], 1);
    vel[pos] = (int)(i / dV);
}
__global__ void k_vinc_sort(const long long *__restrict__ vptr, long long nV, int *__restrict__ vel) {
    long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= nV) return;
    long long b = vptr[v], e = vptr[v + 1];
    for (long long i = b + 1; i < e; i++) {
        int x = vel[i];
        long long j = i - 1;
        while (j >= b && vel[j] > x) { vel[j + 1] = vel[j]; j--; }
        vel[j + 1] = x;
    }
}

constexpr int MAX_ADJ_CAND = 320;

template <int DIM>
__global__ void k_adjacency(const int *__restrict__ T32, long long nE, const long long *__restrict__ vptr,
                            const int *__restrict__ vel, const long long *__restrict__ xadj,
                            int *__restrict__ cnt, int *__restrict__ adj, int *__restrict__ err) {
    constexpr int dV = DIM + 1;
    long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= nE) return;
    int c[MAX_ADJ_CAND];
    int n = 0;
    for (int k = 0; k < dV; k++) {
        int v = T32[e * dV + k];
        for (long long j = vptr[v]; j < vptr[v + 1]; j++) {
            int o = vel[j];
            if (o == (int)e) continue;
            if (n >= MAX_ADJ_CAND) { atomicOr(err, 1); return; }
            // insertion into sorted unique list
            int i = n - 1;
            bool dup = false;
            while (i >= 0 && c[i] >= o) { if (c[i] == o) { dup = true; break; } i--; }
            if (dup) continue;
            for (int t = n; t > i + 1; t--) c[t] = c[t - 1];
            c[i + 1] = o;
            n++;
        }
    }
    if (!adj) { cnt[e] = n; return; }
    long long o = xadj[e];
    for (int i = 0; i < n; i++) adj[o + i] = c[i];
}

// ------------------------------------------------------------------ BFS pair search
constexpr int BFS_THREADS = 256;
constexpr int BFS_WARPS = BFS_THREADS / 32;

struct BfsArgs {
    const int *T32, *labT, *eprob;
    const double *EC;
    const float *EChi, *EClo;
    const float *BCf;        // barycenters, double-float (BC_STRIDE floats per element)
    unsigned long long *n_amb;
    const ProbParams *probs;
    long long nE;
    // Per-warp visited stamps (16-bit): a warp marks what it has met for its current outer element
    // with that element's epoch, a per-warp counter kept across launches in epoch[]. Nothing is
    // cleared between outer elements or assemblies; when a warp's counter wraps, the warp clears
    // its own stamps.
    unsigned short *visited;   // nwarps * vstride: elements
    long long vstride;
    const long long *vptr;     // vertex -> incident elements (sorted)
    const int *vel;
    unsigned short *vvisited;  // nwarps * vvstride: vertices whose incident elements were seen
    long long vvstride;
    unsigned *epoch;           // nwarps: the last epoch each warp used
    int *queue;              // nwarps * qcap
    long long qcap;
    int *pool;               // pool of bT per aT segment
    long long pool_cap;
    unsigned long long *pool_cursor;
    long long *seg_start;
    int *seg_cnt;
    unsigned long long *n_cand;
    unsigned long long *work;   // next outer element to hand out (chunks of BFS_CHUNK)
    int *err;                // [0] queue overflow, [1] pool overflow, [2] bad method
    long long *qneed;
};

// Interaction predicate of integrate(aT, bT) for the configured method: the return value of
// integrate_retriangulate / integrate_baryCenter / integrate_fractional (integration.cpp:539,
// 1017, 287) and of the 2D rules retriangulate_unsymm (:703), subSetBall / averageBall (:1094),
// baryCenterRT (:1247) and noTruncation (:342), OR'ed with is_fullConnectedComponentSearch.
template <int DIM>
__device__ __forceinline__ bool interacts_exact(const ProbParams &P, int method, const double *xs,
                                                int nPx, const double *Ea, const double *Eb) {
    if (P.full_search) return true;
    if (method == MTH_FRACTIONAL || method == MTH_WEAKSING || method == MTH_NOTRUNC) return true;
    if (DIM == 2 && (method == MTH_SUBSET || method == MTH_AVERAGE)) {   // a vertex strictly inside
        for (int k = 0; k < nPx; k++)
            for (int v = 0; v <= DIM; v++)
                if (xsqdist2(&Eb[2 * v], &xs[2 * k]) < P.sqdelta) return true;
        return false;
    }
    if (DIM == 2 && method == MTH_BARY_RT) {   // aT meets the ball around bT's barycenter
        double bc[2], R[18];
        xbary<2>(Eb, bc);
        return xretriangulate(bc, Ea, P.sqdelta, P.caps, R) >= 3;
    }
    if (method == MTH_BARYCENTER) {
        double b[DIM];
        xbary<DIM>(Eb, b);
        for (int k = 0; k < nPx; k++)
            if (xbaryInside<DIM>(&xs[DIM * k], b, P.sqdelta)) return true;
        return false;
    }
    if (DIM == 2) {   // retriangulate, retriangulate_unsymm; exactBall: the polygon without cap points
        double R[18];
        const int caps = method == MTH_EXACT ? 0 : P.caps;
        for (int k = 0; k < nPx; k++)
            if (xretriangulate(&xs[2 * k], Eb, P.sqdelta, caps, R) >= 3) return true;
    }
    return false;
}

// method_baryCenter for some outer point (integrate_baryCenter's doesInteract) with the FP32
// barycenter offset bf; the exact FP64 test decides the points within the squared-distance margin.
// oc holds the outer points' centroid and the radius ro of a sphere around it holding them all: a
// barycenter farther than delta + ro from the centroid is outside every ball (checked with the
// squared-distance margin, ro inflated by 8u).
template <int DIM>
__device__ __forceinline__ bool bary_filtered(const ProbParams &P, const double *xs, const float *xsf, int nPx,
                                              const double *Eb, const float *bf, const float *oc, unsigned &namb) {
    const float sqlo = P.sqdelta_f * (1.f - MARG_D), sqhi = P.sqdelta_f * (1.f + MARG_D);
    {
        float dc = 0.f;
#pragma unroll
        for (int j = 0; j < DIM; j++) { const float d = bf[j] - oc[j]; dc = fmaf(d, d, dc); }
        const float R = sqrtf(P.sqdelta_f) + oc[3];
        if (dc > R * R * (1.f + MARG_D)) return false;
    }
    double b64[DIM];
    bool have_b64 = false;
    for (int k = 0; k < nPx; k++) {
        float d2 = 0.f;
#pragma unroll
        for (int j = 0; j < DIM; j++) { float d = xsf[DIM * k + j] - bf[j]; d2 = fmaf(d, d, d2); }
        if (d2 < sqlo) return true;
        if (d2 > sqhi) continue;
        namb++;
        if (!have_b64) { xbary<DIM>(Eb, b64); have_b64 = true; }
        if (xbaryInside<DIM>(&xs[DIM * k], b64, P.sqdelta)) return true;
    }
    return false;
}

// The same predicate with the certified FP32 geometry (certified.cuh); the exact FP64 routine
// runs only for outer points whose FP32 decisions are within their margins.
template <int DIM>
__device__ __forceinline__ bool interacts_filtered(const ProbParams &P, int method, const double *xs,
                                                   const float *xsf, int nPx, const double *Eb,
                                                   const float *pb, unsigned &namb) {
    if (P.full_search) return true;
    if (method == MTH_FRACTIONAL || method == MTH_WEAKSING) return true;   // close rules: every candidate
    const float sqlo = P.sqdelta_f * (1.f - MARG_D), sqhi = P.sqdelta_f * (1.f + MARG_D);
    if (DIM != 2) return false;
    const F2 p[3] = {f2(pb[0], pb[1]), f2(pb[2], pb[3]), f2(pb[4], pb[5])};
    // First, per outer point, the disc around the triangle's centroid through its farthest vertex:
    // a ball holding that disc holds the triangle (the polygon is the triangle itself: three
    // points), and a ball missing it misses the triangle. Both with the squared-distance margin.
    const F2 cen = f2((p[0].x + p[1].x + p[2].x) * (1.f / 3.f), (p[0].y + p[1].y + p[2].y) * (1.f / 3.f));
    float rb2 = 0.f;
#pragma unroll
    for (int i = 0; i < 3; i++) { const F2 w = p[i] - cen; rb2 = fmaxf(rb2, dot(w, w)); }
    const float rb = sqrtf(rb2) * (1.f + 8.f * U32), dl = sqrtf(P.sqdelta_f);
    const float din = dl - rb;
    const float sq_in = din > 0.f ? din * din * (1.f - MARG_D) : -1.f;
    const float sq_out = (dl + rb) * (dl + rb) * (1.f + MARG_D);
    unsigned und = 0;   // outer points the disc test leaves open
    int kn = 0;
    float dn = 3.0e38f;
    for (int k = 0; k < nPx; k++) {
        const F2 q = cen - f2(xsf[2 * k], xsf[2 * k + 1]);
        const float dc = dot(q, q);
        if (dc < sq_in) return true;
        if (dc > sq_out) continue;
        und |= 1u << k;
        if (dc < dn) { dn = dc; kn = k; }
    }
    if (!und) return false;
    // Then the cheap certain answer, nearest point first: one vertex strictly inside and none on
    // the sphere means both edges through it cross once, so the polygon has at least three
    // points. Only when no point gives it does any point need its polygon.
    unsigned cut = 0;   // outer points whose ball may cut the triangle
    for (unsigned rest = und, first = 1; rest; first = 0) {
        const int k = first ? kn : __ffs(rest) - 1;
        rest &= ~(1u << k);
        const F2 x = f2(xsf[2 * k], xsf[2 * k + 1]);
        const F2 Q[3] = {p[0] - x, p[1] - x, p[2] - x};
        const float d0 = dot(Q[0], Q[0]), d1 = dot(Q[1], Q[1]), d2 = dot(Q[2], Q[2]);
        const bool clear = (d0 < sqlo || d0 > sqhi) && (d1 < sqlo || d1 > sqhi) && (d2 < sqlo || d2 > sqhi);
        if (clear && (d0 < sqlo || d1 < sqlo || d2 < sqlo)) return true;
        if (fclassify(Q, P.sqdelta_f) != CLS_OUT) cut |= 1u << k;
    }
    for (; cut; cut &= cut - 1) {
        const int k = __ffs(cut) - 1;
        const F2 x = f2(xsf[2 * k], xsf[2 * k + 1]);
        const F2 Q[3] = {p[0] - x, p[1] - x, p[2] - x};
        bool amb = false;
        const int n = fretriangulate(Q, P.sqdelta_f, P.caps, nullptr, amb);   // the count only
        if (!amb) {
            if (n >= 3) return true;
            continue;
        }
        namb++;
        double R64[18];
        if (xretriangulate(&xs[2 * k], Eb, P.sqdelta, P.caps, R64) >= 3) return true;
    }
    return false;
}

// Appends val for every lane with push, in lane order.
__device__ __forceinline__ void queue_push(bool push, int val, int *queue, long long qcap, long long &qtail,
                                           bool &overflow) {
    const unsigned m = __ballot_sync(FULL, push);
    if (push) {
        const long long pos = qtail + __popc(m & lanemask_lt());
        if (pos < qcap) queue[pos] = val;
        else overflow = true;
    }
    qtail += __popc(m);
}

// Interaction test of candidate b against the outer element's points (doesInteract of the
// integrate routines, integration.cpp:539,1017).
template <int DIM, int PREC>
__device__ __forceinline__ bool bfs_test(const BfsArgs &a, const ProbParams &P, int method, const double *xs,
                                         const float *xsf, int nPx, const float *ohi, const float *olo,
                                         const double *Ea, int b, const float *oc, unsigned &namb) {
    constexpr int dV = DIM + 1;
    const double *Eb = &a.EC[(long long)b * DIM * dV];
    if (PREC == PREC_F64) return interacts_exact<DIM>(P, method, xs, nPx, Ea, Eb);
    if (method == MTH_BARYCENTER && !P.full_search) {
        float bf[DIM];
        bary_offset<DIM>(a.BCf, b, ohi, olo, bf);
        return bary_filtered<DIM>(P, xs, xsf, nPx, Eb, bf, oc, namb);
    }
    if (DIM != 2) return P.full_search || method == MTH_FRACTIONAL || method == MTH_WEAKSING;
    float pb[DIM * dV];
#pragma unroll
    for (int j = 0; j < DIM * dV; j++)
        pb[j] = (a.EChi[(long long)b * DIM * dV + j] - ohi[j % DIM]) + (a.EClo[(long long)b * DIM * dV + j] - olo[j % DIM]);
    return interacts_filtered<DIM>(P, method, xs, xsf, nPx, Eb, pb, namb);
}

// One warp per outer element aT: breadth-first search over the vertex-sharing element graph from
// aT, through the elements that interact with aT (Cassemble.cpp:597-660).
//   * A group of up to 32 queued elements loads all its vertices at once; each vertex is
//     expanded the first time the search meets it (per-warp vertex stamps).
//   * Each fresh vertex lists its incident elements, BFS_UNROLL entries per lane loaded together;
//     they are then checked one step at a time against the per-warp element stamps (a plain load
//     and store: an element is met from each of its vertices in quick succession, so the stamp is
//     usually in L1). Lanes holding the same element in a step keep only the lowest.
//   * Fresh candidates collect in a per-warp buffer and are tested 32 at a time.
// Without a singular kernel the walk order does not change the result (the connected component
// of aT among interacting elements and label-0 bridges), so the queue is consumed in groups of
// 32 with no level barrier. With one, the candidates found from aT itself (the elements sharing a
// vertex with it) take the close rule and are all tested before the walk goes on.
constexpr int BFS_UNROLL = 4;
// Outer elements are handed out in chunks of consecutive indices (at most BFS_CHUNK, fewer near
// the end): neighbouring elements (in a mesh numbered with any locality) meet largely the same
// candidates, so the warp's stamps of the previous element are still in cache for the next one.
constexpr int BFS_CHUNK = 8;

// 3D searches (barycenter tests, no polygon geometry) fit 64 registers and gain from the doubled
// residency; the 2D retriangulate test needs more.
template <int DIM, int PREC>
__global__ void __launch_bounds__(BFS_THREADS, DIM == 3 ? 4 : 2) k_bfs(BfsArgs a, Rule rule) {
    constexpr int dV = DIM + 1;
    constexpr int U = BFS_UNROLL;
    __shared__ double s_x[BFS_WARPS][MAXQ * DIM];
    __shared__ float s_xf[BFS_WARPS][MAXQ * DIM];
    __shared__ float s_oc[BFS_WARPS][4];                // outer points' centroid and enclosing radius
    __shared__ int s_buf[BFS_WARPS][32 * U + 32];       // candidates waiting for the interaction test
    __shared__ int s_vbuf[BFS_WARPS][32 * (DIM + 1)];   // fresh vertices of a queue group
    unsigned namb = 0;
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const int wpb = blockDim.x >> 5;   // at most BFS_WARPS
    const long long gw = (long long)blockIdx.x * wpb + wib;
    unsigned short *visited = a.visited + gw * a.vstride;
    unsigned short *vvis = a.vvisited + gw * a.vvstride;
    unsigned ep = a.epoch[gw];
    int *vbuf = s_vbuf[wib];
    int *buf = s_buf[wib];
    int *queue = a.queue + gw * a.qcap;
    double *xs = s_x[wib];
    unsigned long long cand_local = 0;
    long long cnext = 0, cend = 0;   // the warp's current chunk of consecutive outer elements
    for (;;) {
        if (cnext == cend) {
            unsigned long long c0 = 0;
            long long ch = 1;
            if (lane == 0) {
                // guided: chunks shrink to one element as the work runs out, so warps finish
                // together (an element of a 2·256² triangle mesh at delta = 0.1 costs a warp about
                // a millisecond); the counter read may be stale, which only changes a chunk's size
                const long long rem = a.nE - (long long)*(volatile unsigned long long *)a.work;
                const long long nw = (long long)gridDim.x * wpb;
                ch = rem / (2 * nw);
                ch = ch < 1 ? 1 : (ch > BFS_CHUNK ? BFS_CHUNK : ch);
                c0 = atomicAdd(a.work, (unsigned long long)ch);
            }
            c0 = __shfl_sync(FULL, c0, 0);
            ch = __shfl_sync(FULL, ch, 0);
            if (c0 >= (unsigned long long)a.nE) break;
            cnext = (long long)c0;
            cend = cnext + ch < a.nE ? cnext + ch : a.nE;
        }
        const long long aT = cnext++;
        const int lab = a.labT[aT];
        if (lab == 0) {
            if (lane == 0) { a.seg_cnt[aT] = 0; a.seg_start[aT] = 0; }
            continue;
        }
        const ProbParams P = a.probs[a.eprob[aT]];
        const long long eoff = P.elem_off;
        const long long voff = P.vert_off;
        ep = (ep + 1u) & 0xffffu;
        if (ep == 0u) {   // the 16-bit epochs wrapped: clear this warp's stamps
            for (long long i = lane; i < a.vstride; i += 32) visited[i] = 0;
            for (long long i = lane; i < a.vvstride; i += 32) vvis[i] = 0;
            __syncwarp();
            ep = 1u;
        }
        const unsigned short stamp = (unsigned short)ep;
        const double *Ea = &a.EC[aT * DIM * dV];
        float ohi[DIM], olo[DIM];
#pragma unroll
        for (int j = 0; j < DIM; j++) { ohi[j] = a.EChi[aT * DIM * dV + j]; olo[j] = a.EClo[aT * DIM * dV + j]; }
        float *xsf = s_xf[wib];
        for (int k = lane; k < rule.nPx; k += 32) {
            xtoPhys<DIM>(Ea, &rule.Px[DIM * k], &xs[DIM * k]);
#pragma unroll
            for (int j = 0; j < DIM; j++) xsf[DIM * k + j] = (float)(xs[DIM * k + j] - Ea[j]);
        }
        __syncwarp();
        if (PREC != PREC_F64 && lane == 0) {
            float c[DIM], r2 = 0.f;
#pragma unroll
            for (int j = 0; j < DIM; j++) {
                float t = 0.f;
                for (int k = 0; k < rule.nPx; k++) t += xsf[DIM * k + j];
                c[j] = t / (float)rule.nPx;
                s_oc[wib][j] = c[j];
            }
            for (int k = 0; k < rule.nPx; k++) {
                float d2 = 0.f;
#pragma unroll
                for (int j = 0; j < DIM; j++) { const float d = xsf[DIM * k + j] - c[j]; d2 = fmaf(d, d, d2); }
                r2 = fmaxf(r2, d2);
            }
            s_oc[wib][3] = sqrtf(r2) * (1.f + 8.f * U32);
        }
        __syncwarp();
        // (aT, aT): the first candidate of the first dequeued element (Cassemble.cpp:621)
        bool self_pair = false;
        if (lane == 0) {
            visited[aT - eoff] = stamp;
            self_pair = interacts_exact<DIM>(P, P.singular ? P.close : P.remote, xs, rule.nPx, Ea, Ea);
            queue[0] = (int)aT;
        }
        self_pair = __shfl_sync(FULL, self_pair, 0);
        __syncwarp();   // aT's stamp and queue entry before any lane reads them
        cand_local += (lane == 0);
        long long qhead = 0, qtail = 1;
        bool overflow = false;
        int nbuf = 0;
        bool lvl0 = true;   // expanding aT itself
        // tests the last cnt (<= 32) buffered candidates and queues those that interact
        auto test_batch = [&](int cnt) {
            const int b = lane < cnt ? buf[nbuf - cnt + lane] : -1;
            __syncwarp();   // read before later appends reuse the slots
            nbuf -= cnt;
            const int method = (P.singular && lvl0) ? P.close : P.remote;
            bool pair = false;
            if (b >= 0) {
                pair = bfs_test<DIM, PREC>(a, P, method, xs, xsf, rule.nPx, ohi, olo, Ea, b, s_oc[wib], namb);
                cand_local++;
            }
            queue_push(pair, b, queue, a.qcap, qtail, overflow);
        };
        for (;;) {
            const long long avail = qtail - qhead;
            if (avail > 0 && (avail >= 32 || nbuf == 0 || lvl0)) {
                const int gn = (int)(avail < 32 ? avail : 32);
                int sn = lane < gn ? queue[qhead + lane] : -1;
                qhead += gn;
                if (sn < -1) sn = -sn - 2;   // label-0 bridge stored as -(e+2)
                int vv[dV];
#pragma unroll
                for (int r = 0; r < dV; r++) vv[r] = sn >= 0 ? a.T32[(long long)sn * dV + r] : -1;
                int nv = 0;
#pragma unroll
                for (int r = 0; r < dV; r++) {
                    int v = vv[r];
                    const unsigned same = __match_any_sync(FULL, v);
                    if ((__ffs(same) - 1) != lane) v = -1;
                    bool fresh = false;
                    if (v >= 0) {
                        fresh = vvis[v - voff] != stamp;
                        if (fresh) vvis[v - voff] = stamp;
                    }
                    const unsigned m = __ballot_sync(FULL, fresh);
                    if (fresh) vbuf[nv + __popc(m & lanemask_lt())] = v;
                    nv += __popc(m);
                    __syncwarp();   // the stamps of this round before the next round's loads
                }
                for (int c0 = 0; c0 < nv; c0 += 32) {
                    const int v = c0 + lane < nv ? vbuf[c0 + lane] : -1;
                    long long beg = 0;
                    int deg = 0;
                    if (v >= 0) { beg = a.vptr[v]; deg = (int)(a.vptr[v + 1] - beg); }
                    const int maxdeg = (int)__reduce_max_sync(FULL, (unsigned)deg);
                    for (int j0 = 0; j0 < maxdeg; j0 += U) {
                        int cand[U];
#pragma unroll
                        for (int u = 0; u < U; u++) cand[u] = j0 + u < deg ? a.vel[beg + j0 + u] : -1;
#pragma unroll
                        for (int u = 0; u < U; u++) {
                            int c = cand[u];
                            const int lb = (P.bridges && c >= 0) ? a.labT[c] : 1;
                            // lanes holding the same element: the lowest takes it
                            const unsigned same = __match_any_sync(FULL, c);
                            if ((__ffs(same) - 1) != lane) c = -1;
                            bool fresh = false;
                            if (c >= 0) {
                                fresh = visited[c - eoff] != stamp;
                                if (fresh) visited[c - eoff] = stamp;
                            }
                            const bool bridge = fresh && lb == 0;
                            queue_push(bridge, -(c + 2), queue, a.qcap, qtail, overflow);
                            const bool totest = fresh && !bridge;
                            const unsigned m = __ballot_sync(FULL, totest);
                            if (totest) buf[nbuf + __popc(m & lanemask_lt())] = c;
                            nbuf += __popc(m);
                            __syncwarp();   // this step's stamps before the next step's loads
                        }
                        while (nbuf >= 32) test_batch(32);
                    }
                }
                if (lvl0) {   // the close candidates are tested before the walk goes on
                    while (nbuf > 0) test_batch(nbuf < 32 ? nbuf : 32);
                    lvl0 = false;
                }
            } else if (nbuf > 0) {
                test_batch(nbuf < 32 ? nbuf : 32);
            } else {
                break;
            }
            if (__any_sync(FULL, overflow)) break;
        }
        overflow = __any_sync(FULL, overflow);
        if (overflow) {
            if (lane == 0) {
                atomicOr(&a.err[0], 1);
                atomicMax((unsigned long long *)a.qneed, (unsigned long long)(qtail + 1));
                a.seg_cnt[aT] = 0;
                a.seg_start[aT] = 0;
            }
            continue;
        }
        // pairs: queue entries that interacted (queue[0] = aT only if (aT, aT) interacts)
        int npairs = 0;
        for (long long g = 0; g < qtail; g += 32) {
            long long gi = g + lane;
            bool isp = false;
            if (gi < qtail) {
                int s = queue[gi];
                isp = (gi == 0) ? self_pair : (s >= 0);
            }
            npairs += __popc(__ballot_sync(FULL, isp));
        }
        unsigned long long base = 0;
        if (lane == 0) base = atomicAdd(a.pool_cursor, (unsigned long long)npairs);
        base = __shfl_sync(FULL, base, 0);
        const bool fits = base + npairs <= (unsigned long long)a.pool_cap;
        if (lane == 0) {
            a.seg_cnt[aT] = npairs;
            a.seg_start[aT] = (long long)base;
            if (!fits) atomicOr(&a.err[1], 1);
        }
        if (fits) {
            int w = 0;
            for (long long g = 0; g < qtail; g += 32) {
                long long gi = g + lane;
                bool isp = false;
                int s = -1;
                if (gi < qtail) {
                    s = queue[gi];
                    isp = (gi == 0) ? self_pair : (s >= 0);
                }
                const unsigned m = __ballot_sync(FULL, isp);
                if (isp) a.pool[base + w + __popc(m & lanemask_lt())] = s;
                w += __popc(m);
            }
        }
    }
    if (lane == 0) a.epoch[gw] = ep;
    cand_local = warp_sum(cand_local);
    if (lane == 0 && cand_local) atomicAdd(a.n_cand, cand_local);
    namb = warp_sum(namb);
    if (lane == 0 && namb && a.n_amb) atomicAdd(a.n_amb, (unsigned long long)namb);
}

// aT-major compaction of the BFS segments.
__global__ void k_compact_pairs(const long long *__restrict__ seg_start, const int *__restrict__ seg_cnt,
                                const long long *__restrict__ out_ptr, const int *__restrict__ pool,
                                long long nE, int *__restrict__ pA, int *__restrict__ pB) {
    const int lane = threadIdx.x & 31;
    long long e = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (e >= nE) return;
    const int n = seg_cnt[e];
    const long long s = seg_start[e], o = out_ptr[e];
    for (int i = lane; i < n; i += 32) {
        pA[o + i] = (int)e;
        pB[o + i] = pool[s + i];
    }
}

__global__ void k_in_count(const int *__restrict__ pB, long long P, int *__restrict__ incnt) {
    long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (p < P) atomicAdd(&incnt[pB[p]], 1);
}
__global__ void k_in_fill(const int *__restrict__ pA, const int *__restrict__ pB, long long P,
                          const long long *__restrict__ in_ptr, int *__restrict__ infill,
                          int *__restrict__ inA) {
    long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= P) return;
    int b = pB[p];
    long long pos = in_ptr[b] + atomicAdd(&infill[b], 1);
    inA[pos] = pA[p];
}

// ------------------------------------------------------------------ CSR pattern
struct RowArgs {
    const int *T32, *labT, *labV, *vprob, *vel, *pB, *inA;
    const long long *vptr, *out_ptr, *in_ptr;
    const int *out_cnt;        // out-pair counts when the out-lists are pool segments (see PassArgs)
    const ProbParams *probs;
    long long nV;
    unsigned *marks;       // nwarps * mstride
    long long mstride;
    const long long *rowptr;   // fill mode
    int *cols;                 // fill mode (null: count mode)
    int *rowcnt;               // count mode
    // direct mode (bitmap kernel, pass 2): rows placed in scratch at an atomic cursor
    int *scratch;
    long long cap;             // scratch capacity (ints)
    unsigned long long *cursor;
    long long *rowoff;         // scratch offset of each row
    int *ovf;                  // set when the scratch is too small
    // bitmap kernel sources: mode 0, the vertices of the pairs of the elements at the row's
    // vertex (rows of vertices with label > 0, or of every vertex with all_rows); mode 1, the
    // union of a given row (srcoff / srccnt / srccols) and a given transposed row (tptr / tcols);
    // mode 2, the same rows as mode 0 for one-sided passes (out-pairs only) as the union of the
    // rows' elements' vertex lists (vpool / vseg_start / vseg_cnt: mode 0 run over elements, each
    // element its own row, lists its partners' vertices and its own)
    int mode, all_rows;
    const int *vpool;
    const long long *vseg_start;
    const int *vseg_cnt;
    const long long *srcoff;
    const int *srccnt, *srccols;
    const long long *tptr;
    const int *tcols;
};

// One warp per row (vertex) u with label > 0: union of the vertices of every element that
// shares a pair with an element incident to u.
template <int DIM>
__global__ void __launch_bounds__(256) k_row_pattern(RowArgs a, int pass) {
    constexpr int dV = DIM + 1;
    const int lane = threadIdx.x & 31;
    const long long gw = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const long long nw = ((long long)gridDim.x * blockDim.x) >> 5;
    unsigned *marks = a.marks + gw * a.mstride;
    for (long long u = gw; u < a.nV; u += nw) {
        const bool keep = a.labV[u] > 0;
        if (!keep) {
            if (!a.cols && lane == 0) a.rowcnt[u] = 0;
            continue;
        }
        const int voff = a.probs[a.vprob[u]].vert_off;
        const unsigned stamp = (unsigned)(2 * u + 1 + pass);   // unique per row and pass
        long long w = 0;
        const long long rbase = a.cols ? a.rowptr[u] : 0;
        for (long long t = a.vptr[u]; t < a.vptr[u + 1]; t++) {
            const int T = a.vel[t];
            const long long ob = a.out_ptr[T], oe = a.out_cnt ? ob + a.out_cnt[T] : a.out_ptr[T + 1];
            const long long ib = a.in_ptr ? a.in_ptr[T] : 0, ie = a.in_ptr ? a.in_ptr[T + 1] : 0;
            if (oe == ob && ie == ib) continue;
            const long long nEl = 1 + (oe - ob) + (ie - ib);
            const long long nItems = nEl * dV;
            for (long long i0 = 0; i0 < nItems; i0 += 32) {
                const long long i = i0 + lane;
                bool isnew = false;
                int v = 0;
                if (i < nItems) {
                    const long long el_i = i / dV;
                    const int k = (int)(i - el_i * dV);
                    int el;
                    if (el_i == 0) el = T;
                    else if (el_i <= oe - ob) el = a.pB[ob + el_i - 1];
                    else el = a.inA[ib + (el_i - 1 - (oe - ob))];
                    v = a.T32[(long long)el * dV + k];
                    unsigned old = atomicExch(&marks[v - voff], stamp);
                    isnew = old != stamp;
                }
                const unsigned m = __ballot_sync(FULL, isnew);
                if (a.cols && isnew) a.cols[rbase + w + __popc(m & lanemask_lt())] = v;
                w += __popc(m);
            }
        }
        if (!a.cols && lane == 0) a.rowcnt[u] = (int)w;
    }
}

// Same row sets with the marks as a bitmap over the problem's vertices in shared memory (words
// 32-bit words per warp): a shared-memory atomicOr replaces the global exchange, and the set
// bits come out in increasing order, so the rows need no sort. pass 0 counts, pass 1 writes.
template <int DIM>
__global__ void __launch_bounds__(256) k_row_pattern_bm(RowArgs a, int pass, int words) {
    extern __shared__ unsigned s_bm[];
    constexpr int dV = DIM + 1;
    const int lane = threadIdx.x & 31;
    unsigned *bm = s_bm + (size_t)(threadIdx.x >> 5) * words;
    const long long gw = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const long long nw = ((long long)gridDim.x * blockDim.x) >> 5;
    // the bitmap is cleared once here; each row clears the words it touched when it is done
    for (int i = lane; i < words; i += 32) bm[i] = 0u;
    __syncwarp();
    for (long long u = gw; u < a.nV; u += nw) {
        if (!a.all_rows && a.labV[u] <= 0) {
            if (pass != 1 && lane == 0) a.rowcnt[u] = 0;
            if (pass == 2 && lane == 0) a.rowoff[u] = 0;
            continue;
        }
        const ProbParams &P = a.probs[a.vprob[u]];
        const int voff = P.vert_off;
        int lo = 0x7fffffff, hi = -1;
        if (a.mode == 1) {   // union of a row and its transposed row
            const long long o = a.srcoff[u];
            const int n = a.srccnt[u];
            for (int i = lane; i < n; i += 32) {
                const int v = a.srccols[o + i] - voff;
                atomicOr(&bm[v >> 5], 1u << (v & 31));
                lo = min(lo, v);
                hi = max(hi, v);
            }
            for (long long i = a.tptr[u] + lane; i < a.tptr[u + 1]; i += 32) {
                const int v = a.tcols[i] - voff;
                atomicOr(&bm[v >> 5], 1u << (v & 31));
                lo = min(lo, v);
                hi = max(hi, v);
            }
        }
        if (a.mode == 2) {   // union of the vertex lists of the elements at u
            for (long long t = a.vptr[u]; t < a.vptr[u + 1]; t++) {
                const int T = a.vel[t];
                const long long b = a.vseg_start[T];
                const int n = a.vseg_cnt[T];
                for (int i = lane; i < n; i += 32) {
                    const int v = a.vpool[b + i] - voff;
                    atomicOr(&bm[v >> 5], 1u << (v & 31));
                    lo = min(lo, v);
                    hi = max(hi, v);
                }
            }
        }
        for (long long t = a.mode != 0 ? a.vptr[u + 1] : a.vptr[u]; t < a.vptr[u + 1]; t++) {
            const int T = a.vel[t];
            const long long ob = a.out_ptr[T], oe = a.out_cnt ? ob + a.out_cnt[T] : a.out_ptr[T + 1];
            const long long ib = a.in_ptr ? a.in_ptr[T] : 0, ie = a.in_ptr ? a.in_ptr[T + 1] : 0;
            if (oe == ob && ie == ib) continue;
            const int nout = (int)(oe - ob), nEl = 1 + nout + (int)(ie - ib);
            for (int el_i = lane; el_i < nEl; el_i += 32) {   // one partner element per lane
                int el;
                if (el_i == 0) el = T;
                else if (el_i <= nout) el = a.pB[ob + el_i - 1];
                else el = a.inA[ib + (el_i - 1 - nout)];
#pragma unroll
                for (int k = 0; k < dV; k++) {
                    const int v = a.T32[(long long)el * dV + k] - voff;
                    atomicOr(&bm[v >> 5], 1u << (v & 31));
                    lo = min(lo, v);
                    hi = max(hi, v);
                }
            }
        }
        __syncwarp();
        lo = __reduce_min_sync(FULL, lo);
        hi = __reduce_max_sync(FULL, hi);
        if (pass == 2) {   // direct: count, take scratch space, write the sorted columns there
            int cnt = 0;
            if (hi >= 0)
                for (int wi = (lo >> 5) + lane; wi <= (hi >> 5); wi += 32) cnt += __popc(bm[wi]);
            cnt = warp_sum(cnt);
            unsigned long long off = 0;
            if (lane == 0) {
                off = atomicAdd(a.cursor, (unsigned long long)cnt);
                a.rowcnt[u] = cnt;
                a.rowoff[u] = (long long)off;
                if ((long long)off + cnt > a.cap) atomicOr(a.ovf, 1);
            }
            off = __shfl_sync(FULL, off, 0);
            if (hi >= 0 && (long long)off + cnt <= a.cap) {
                long long w = (long long)off;
                for (int w0 = lo >> 5; w0 <= (hi >> 5); w0 += 32) {
                    const int wi = w0 + lane;
                    unsigned bits = wi <= (hi >> 5) ? bm[wi] : 0u;
                    const int c = __popc(bits);
                    const int incl = warp_incl_scan(c, lane);
                    long long o = w + incl - c;
                    while (bits) {
                        const int b = __ffs(bits) - 1;
                        a.scratch[o++] = voff + wi * 32 + b;
                        bits &= bits - 1;
                    }
                    w += __shfl_sync(FULL, incl, 31);
                }
            }
            __syncwarp();
            if (hi >= 0)
                for (int wi = (lo >> 5) + lane; wi <= (hi >> 5); wi += 32) bm[wi] = 0u;
            __syncwarp();
            continue;
        }
        long long w = pass ? a.rowptr[u] : 0;
        if (hi >= 0) {
            for (int w0 = lo >> 5; w0 <= (hi >> 5); w0 += 32) {
                const int wi = w0 + lane;
                unsigned bits = wi <= (hi >> 5) ? bm[wi] : 0u;
                const int c = __popc(bits);
                const int incl = warp_incl_scan(c, lane);
                if (pass) {
                    long long o = w + incl - c;
                    while (bits) {
                        const int b = __ffs(bits) - 1;
                        a.cols[o++] = voff + wi * 32 + b;
                        bits &= bits - 1;
                    }
                }
                w += __shfl_sync(FULL, incl, 31);
            }
        }
        if (pass == 0 && lane == 0) a.rowcnt[u] = (int)w;
        __syncwarp();
        if (hi >= 0)
            for (int wi = (lo >> 5) + lane; wi <= (hi >> 5); wi += 32) bm[wi] = 0u;
        __syncwarp();
    }
}

// Identity incidence (row e holds element e alone): rows of the bitmap kernel over elements.
__global__ void k_iota_rows(long long n, long long *__restrict__ ptr, int *__restrict__ idx) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i <= n) ptr[i] = i;
    if (i < n) idx[i] = (int)i;
}

// Transposed rows of the out-pair rows (warp per source row u, its entries in the scratch):
// k_tcount counts, for every column v with a matrix row, the rows u holding it; k_tfill lists them
// (in atomic order: the union pass sorts).
__global__ void k_tcount(const long long *__restrict__ off, const int *__restrict__ cnt,
                         const int *__restrict__ cols, const int *__restrict__ labV, long long nV,
                         int *__restrict__ tcnt) {
    const int lane = threadIdx.x & 31;
    const long long gw = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const long long nw = ((long long)gridDim.x * blockDim.x) >> 5;
    for (long long u = gw; u < nV; u += nw) {
        const long long o = off[u];
        const int n = cnt[u];
        for (int i = lane; i < n; i += 32) {
            const int v = cols[o + i];
            if (labV[v] > 0) atomicAdd(&tcnt[v], 1);
        }
    }
}
__global__ void k_tfill(const long long *__restrict__ off, const int *__restrict__ cnt,
                        const int *__restrict__ cols, const int *__restrict__ labV, long long nV,
                        const long long *__restrict__ tptr, int *__restrict__ tfill, int *__restrict__ tcols) {
    const int lane = threadIdx.x & 31;
    const long long gw = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const long long nw = ((long long)gridDim.x * blockDim.x) >> 5;
    for (long long u = gw; u < nV; u += nw) {
        const long long o = off[u];
        const int n = cnt[u];
        for (int i = lane; i < n; i += 32) {
            const int v = cols[o + i];
            if (labV[v] > 0) tcols[tptr[v] + atomicAdd(&tfill[v], 1)] = (int)u;
        }
    }
}

// Direct mode, second step: each row's columns from the scratch into CSR order (one warp per row).
__global__ void k_row_copy(const long long *__restrict__ rowptr, const long long *__restrict__ rowoff,
                           long long nV, const int *__restrict__ scratch, int *__restrict__ cols) {
    const int lane = threadIdx.x & 31;
    const long long gw = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const long long nw = ((long long)gridDim.x * blockDim.x) >> 5;
    for (long long u = gw; u < nV; u += nw) {
        const long long b = rowptr[u], n = rowptr[u + 1] - b, o = rowoff[u];
        for (long long i = lane; i < n; i += 32) cols[b + i] = scratch[o + i];
    }
}

// Sort each row's columns (bitonic network in shared memory, padded with INT_MAX).
__global__ void k_row_sort(const long long *__restrict__ rowptr, long long nV, int *__restrict__ cols,
                           int cap) {
    extern __shared__ int sh[];
    for (long long u = blockIdx.x; u < nV; u += gridDim.x) {
        const long long b = rowptr[u];
        const int n = (int)(rowptr[u + 1] - b);
        if (n <= 1) continue;
        int n2 = 1;
        while (n2 < n) n2 <<= 1;
        int *s = (n2 <= cap) ? sh : nullptr;
        if (!s) continue;  // longer rows are sorted by k_row_sort_global
        for (int i = threadIdx.x; i < n2; i += blockDim.x) s[i] = i < n ? cols[b + i] : 0x7fffffff;
        __syncthreads();
        for (int k = 2; k <= n2; k <<= 1) {
            for (int j = k >> 1; j > 0; j >>= 1) {
                for (int i = threadIdx.x; i < n2; i += blockDim.x) {
                    int ixj = i ^ j;
                    if (ixj > i) {
                        int x = s[i], y = s[ixj];
                        bool up = (i & k) == 0;
                        if ((x > y) == up) { s[i] = y; s[ixj] = x; }
                    }
                }
                __syncthreads();
            }
        }
        for (int i = threadIdx.x; i < n; i += blockDim.x) cols[b + i] = s[i];
        __syncthreads();
    }
}
// Fallback for rows longer than the shared-memory cap: odd-even transposition in global memory.
__global__ void k_row_sort_global(const long long *__restrict__ rowptr, long long nV,
                                  int *__restrict__ cols, int cap) {
    for (long long u = blockIdx.x; u < nV; u += gridDim.x) {
        const long long b = rowptr[u];
        const int n = (int)(rowptr[u + 1] - b);
        int n2 = 1;
        while (n2 < n) n2 <<= 1;
        if (n <= 1 || n2 <= cap) continue;
        for (int phase = 0; phase < n; phase++) {
            for (int i = 2 * threadIdx.x + (phase & 1); i + 1 < n; i += 2 * blockDim.x) {
                int x = cols[b + i], y = cols[b + i + 1];
                if (x > y) { cols[b + i] = y; cols[b + i + 1] = x; }
            }
            __syncthreads();
        }
    }
}

// ------------------------------------------------------------------ finish
// Per row: number of entries whose FP64 sum is not exactly zero (arma::sp_mat drops the zeros).
// With touched (mixed precision) a slot that received a contribution is kept even when its
// FP32-derived sum cancelled to exactly zero: its exact value is a nonzero below FP32 resolution.
enum { VAL_F64 = 0, VAL_DF = 1, VAL_FX = 2 };
struct FinishArgs {
    int vmode;                       // how the slots hold their sums
    const unsigned char *touched;    // VAL_DF: slots that received a contribution
    const int *vprob;                // VAL_FX: problem of each row (fixed-point unit)
    const ProbParams *probs;
};
// Value of slot i of row u; keep says whether the slot survives (the reference drops exact
// zeros; slots of the mixed passes are kept when they received any contribution).
__device__ __forceinline__ double slot_value(const FinishArgs &f, const double *vals, long long u, long long i,
                                             bool &keep) {
    double v;
    if (f.vmode == VAL_FX) {
        v = (double)reinterpret_cast<const long long *>(vals)[i] * f.probs[f.vprob[u]].fx_unit;
        keep = true;
    } else if (f.vmode == VAL_DF) {
        v = df_to_double(reinterpret_cast<const DF *>(vals)[i]);
        keep = (v != 0.0) || f.touched[i];
    } else {
        v = vals[i];
        keep = v != 0.0;
    }
    return v;
}
__global__ void k_finish_count(const long long *__restrict__ rowptr, long long nV,
                               const double *__restrict__ vals, FinishArgs f, int *__restrict__ keepcnt) {
    const int lane = threadIdx.x & 31;
    long long u = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (u >= nV) return;
    const long long b = rowptr[u], e = rowptr[u + 1];
    int cnt = 0;
    for (long long i = b + lane; i < e; i += 32) {
        bool k;
        slot_value(f, vals, u, i, k);
        cnt += k;
    }
    cnt = warp_sum(cnt);
    if (lane == 0) keepcnt[u] = cnt;
}
__global__ void k_finish_compact(const long long *__restrict__ rowptr, long long nV,
                                 const int *__restrict__ cols, const double *__restrict__ vals,
                                 FinishArgs f, const long long *__restrict__ fptr, int *__restrict__ fcols,
                                 double *__restrict__ fvals) {
    const int lane = threadIdx.x & 31;
    long long u = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (u >= nV) return;
    const long long b = rowptr[u], e = rowptr[u + 1];
    long long w = fptr[u];
    for (long long i0 = b; i0 < e; i0 += 32) {
        long long i = i0 + lane;
        bool k = false;
        double v = 0.0;
        if (i < e) v = slot_value(f, vals, u, i, k);
        unsigned m = __ballot_sync(FULL, k);
        if (k) {
            long long o = w + __popc(m & lanemask_lt());
            fcols[o] = cols[i];
            fvals[o] = v;
        }
        w += __popc(m);
    }
}

// ------------------------------------------------------------------ load vector
// par_forcing / compute_f (Cassemble.cpp:857-928, 149-164)
template <int DIM>
__global__ void k_forcing(const double *__restrict__ EC, const double *__restrict__ adet,
                          const int *__restrict__ labT, const int *__restrict__ T32,
                          const int *__restrict__ labV, const int *__restrict__ eprob,
                          const ProbParams *__restrict__ probs, long long nE, Rule rule,
                          const long long *__restrict__ zptr, const long long *__restrict__ zidx,
                          unsigned long long *__restrict__ facc, unsigned *__restrict__ tiny) {
    constexpr int dV = DIM + 1;
    long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= nE || labT[e] <= 0) return;
    const ProbParams &P = probs[eprob[e]];
    const double *E = &EC[e * DIM * dV];
    double termf[dV];
#pragma unroll
    for (int a = 0; a < dV; a++) termf[a] = 0;
    for (int i = 0; i < rule.nPx; i++) {
        double x[DIM];
        xtoPhys<DIM>(E, &rule.Px[DIM * i], x);
        const double fv = load_f64(P.load, x);
#pragma unroll
        for (int a = 0; a < dV; a++) termf[a] += rule.psix[dV * i + a] * fv * adet[e] * rule.dx[i];
    }
    // domain decomposition: 1 / zeta of the element with itself (Cassemble.cpp:901-908)
    const double w = P.zeta ? zeta_weight(zptr, zidx, e, e) : 1.0;
#pragma unroll
    for (int a = 0; a < dV; a++) {
        int v = T32[e * dV + a];
        if (labV[v] > 0) fx_atomic_add(&facc[2 * (long long)v], termf[a] * w, P.scale_exp, &tiny[v]);
    }
}
// Load vector entries r = od v + o from their fixed-point sums.
__global__ void k_forcing_finish(const unsigned long long *__restrict__ facc, long long K, int od,
                                 const int *__restrict__ vprob, const ProbParams *__restrict__ probs,
                                 double *__restrict__ fd) {
    long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= K) return;
    fd[r] = fx_to_double(facc[2 * r], facc[2 * r + 1], probs[vprob[r / od]].scale_exp);
}

// ------------------------------------------------------------------ geometry debug hooks
__global__ void k_retri_batch(long long n, const double *__restrict__ x, const double *__restrict__ TE,
                              double sqdelta, int caps, int *__restrict__ counts, double *__restrict__ out) {
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double R[18];
    double xc[2] = {x[2 * i], x[2 * i + 1]};
    double E[6];
    for (int j = 0; j < 6; j++) E[j] = TE[6 * i + j];
    int Rdx = xretriangulate(xc, E, sqdelta, caps, R);
    int nt = Rdx < 3 ? 0 : Rdx - 2;
    counts[i] = nt;
    double *o = &out[54 * i];
    for (int k = 0; k < nt; k++)
        for (int c = 0; c < 2; c++) {
            o[2 * (3 * k + 0) + c] = R[c];
            o[2 * (3 * k + 1) + c] = R[2 * (k + 1) + c];
            o[2 * (3 * k + 2) + c] = R[2 * (k + 2) + c];
        }
}
// Certified FP32 retriangulation on the same cases (test hook): count, ambiguity flag, points
// relative to the center.
__global__ void k_retri_cert_batch(long long n, const double *__restrict__ x, const double *__restrict__ TE,
                                   double sqdelta, int caps, int *__restrict__ counts,
                                   int *__restrict__ amb, double *__restrict__ out) {
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    F2 Q[3];
    for (int j = 0; j < 3; j++) Q[j] = f2((float)(TE[6 * i + 2 * j] - x[2 * i]), (float)(TE[6 * i + 2 * j + 1] - x[2 * i + 1]));
    F2 R[9];
    bool a = false;
    unsigned why = 0;
    const int c = fretriangulate(Q, (float)sqdelta, caps, R, a, &why);
    counts[i] = c;
    amb[i] = a ? (int)why | (int)0x100 : 0;
    for (int j = 0; j < c && j < 9; j++) {
        out[18 * i + 2 * j] = R[j].x;
        out[18 * i + 2 * j + 1] = R[j].y;
    }
}

__global__ void k_geom_misc(int op, const double *__restrict__ A, const double *__restrict__ b, int dim,
                            double *__restrict__ out, int *__restrict__ ok) {
    if (threadIdx.x || blockIdx.x) return;
    if (op == 0) { *ok = xtoRef(A, b, out); }
    else if (op == 1) {
        if (dim == 2) xtoPhys<2>(A, b, out); else xtoPhys<3>(A, b, out);
        *ok = 1;
    } else { *ok = xsolve2x2(A, b, out); }
}

}  // namespace nlg

#include "pipeline.inl"
