// Mixed-precision 2D retriangulate pass with per-warp work compaction.
//
// Same contract as k_pass (passes.cuh): one warp per element T of a color, all contributions to
// the rows of T's vertices, deterministic FP64 accumulation. The quadrature work is reorganised
// so the 32 lanes stay busy: for each batch of 32 pairs, every lane classifies its pair's outer
// points (ball contains the element / misses it / cuts it); the (pair, outer point) items are then
// compacted into an "inside" list and a "cut" list and processed 32 at a time, each item writing
// its inner sums to its own shared-memory slot; the owning lane finally folds the slots into the
// pair's local blocks in a fixed order.
#pragma once
#include "passes.cuh"

namespace nlg {

constexpr int MIX_WARPS = 4;
constexpr int MIX_THREADS = 32 * MIX_WARPS;

// Per-warp shared scratch; nPx-dependent arrays follow the struct in dynamic shared memory.
struct MixWarp {
    double x64[MAXQ * 2];   // outer points of T (FP64, exact)
    F2 xf[MAXQ];            // outer points of T, local
    F2 yT[MAXQ];            // inner points of T, local
    float pc[32][6];        // partner element, local coordinates
    float prt[32];          // partner |det|
    int pid[32];            // partner element
    int nitems[2];
};
__host__ __device__ constexpr size_t mix_warp_bytes(int nPx) {
    // MixWarp + res[32][nPx][9] floats + lists[2][32 * nPx] shorts
    return ((sizeof(MixWarp) + 15) / 16) * 16 + (size_t)32 * nPx * 9 * 4 + (size_t)2 * 32 * nPx * 2 + 16;
}

// Inner sums of one "inside" item of the out side: the ball contains bT.
__device__ __forceinline__ void item_out_in(const ProbParams &P, const Rule &rule, const PassRule &pr,
                                            const float *pc, float rT, F2 x, float *res) {
    const F2 p0 = f2(pc[0] - x.x, pc[1] - x.y);
    const F2 e1 = f2(pc[2] - pc[0], pc[3] - pc[1]), e2 = f2(pc[4] - pc[0], pc[5] - pc[1]);
    float iL = 0.f, i0 = 0.f, i1 = 0.f, i2 = 0.f;
    for (int i = 0; i < rule.nPy; i++) {
        const float px = rule.Pyf[2 * i], py = rule.Pyf[2 * i + 1];
        const float yx = p0.x + e1.x * px + e2.x * py;
        const float yy = p0.y + e1.y * px + e2.y * py;
        const float kw = kernel_f32(P, -yx, -yy) * rT;
        iL = fmaf(kw, rule.dyf[i], iL);
        i0 = fmaf(kw, pr.cy[3 * i + 0], i0);
        i1 = fmaf(kw, pr.cy[3 * i + 1], i1);
        i2 = fmaf(kw, pr.cy[3 * i + 2], i2);
    }
    res[0] = iL; res[1] = i0; res[2] = i1; res[3] = i2;
}

// Inner sums of one "cut" item of the out side: polygon of B(x) and bT (certified FP32, exact
// fallback), fan sub-triangles, basis of bT by the inverse affine map.
__device__ __forceinline__ void item_out_cut(const ProbParams &P, const Rule &rule, const float *pc,
                                             F2 x, const double *x64, const double *Eb64,
                                             float *res, unsigned &nsub, unsigned &namb) {
    const F2 Q[3] = {f2(pc[0] - x.x, pc[1] - x.y), f2(pc[2] - x.x, pc[3] - x.y), f2(pc[4] - x.x, pc[5] - x.y)};
    const F2 e1 = Q[1] - Q[0], e2 = Q[2] - Q[0];
    const float idet = 1.f / (e1.x * e2.y - e1.y * e2.x);
    F2 R[9];
    const int n = cut_polygon(Q, P.sqdelta_f, P, x64, Eb64, R, namb);
    float iL = 0.f, i0 = 0.f, i1 = 0.f, i2 = 0.f;
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
            i0 = fmaf(kw, 1.f - r0 - r1, i0);
            i1 = fmaf(kw, r0, i1);
            i2 = fmaf(kw, r1, i2);
        }
    }
    res[0] = iL; res[1] = i0; res[2] = i1; res[3] = i2;
}

// In side items: outer point x of the partner aT, inner element T (local tl, inner points yT).
__device__ __forceinline__ void item_in_in(const ProbParams &P, const Rule &rule, const PassRule &pr,
                                           const F2 *yT, float rTT, F2 x, float *res) {
    float i0 = 0.f, i1 = 0.f, i2 = 0.f;
    float lp[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    for (int i = 0; i < rule.nPy; i++) {
        const F2 y = yT[i] - x;
        const float kw = kernel_f32(P, -y.x, -y.y) * rTT;
        i0 = fmaf(kw, pr.cy[3 * i + 0], i0);
        i1 = fmaf(kw, pr.cy[3 * i + 1], i1);
        i2 = fmaf(kw, pr.cy[3 * i + 2], i2);
#pragma unroll
        for (int ab = 0; ab < 6; ab++) lp[ab] = fmaf(kw, pr.cyy[6 * i + ab], lp[ab]);
    }
    res[0] = i0; res[1] = i1; res[2] = i2;
#pragma unroll
    for (int ab = 0; ab < 6; ab++) res[3 + ab] = lp[ab];
}

__device__ __forceinline__ void item_in_cut(const ProbParams &P, const Rule &rule, const F2 *tl, F2 x,
                                            const double *Ea64, int k, const double *ET64, float *res,
                                            unsigned &nsub, unsigned &namb) {
    const F2 Q[3] = {tl[0] - x, tl[1] - x, tl[2] - x};
    const F2 e1 = Q[1] - Q[0], e2 = Q[2] - Q[0];
    const float idet = 1.f / (e1.x * e2.y - e1.y * e2.x);
    F2 R[9];
    bool amb = false;
    int n = fretriangulate(Q, P.sqdelta_f, P.caps, R, amb);
    if (amb) {
        namb++;
        double x64[2], R64[18];
        xtoPhys<2>(Ea64, &rule.Px[2 * k], x64);
        n = xretriangulate(x64, ET64, P.sqdelta, P.caps, R64);
        for (int j = 0; j < n; j++) R[j] = f2((float)(R64[2 * j] - x64[0]), (float)(R64[2 * j + 1] - x64[1]));
    }
    float i0 = 0.f, i1 = 0.f, i2 = 0.f;
    float lp[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    for (int r = 0; r + 2 < n; r++) {
        const F2 A = R[0], B = R[r + 1] - R[0], C = R[r + 2] - R[0];
        const float rT = fabsf(B.x * C.y - B.y * C.x);
        for (int i = 0; i < rule.nPy; i++) {
            const float qx = rule.Pyf[2 * i], qy = rule.Pyf[2 * i + 1];
            const float yx = A.x + B.x * qx + C.x * qy;
            const float yy = A.y + B.y * qx + C.y * qy;
            const float kw = kernel_f32(P, -yx, -yy) * rT * rule.dyf[i];
            const float dxr = yx - Q[0].x, dyr = yy - Q[0].y;
            const float r0 = (e2.y * dxr - e2.x * dyr) * idet;
            const float r1 = (e1.x * dyr - e1.y * dxr) * idet;
            const float s0 = 1.f - r0 - r1;
            i0 = fmaf(kw, s0, i0);
            i1 = fmaf(kw, r0, i1);
            i2 = fmaf(kw, r1, i2);
            lp[0] = fmaf(kw, s0 * s0, lp[0]); lp[1] = fmaf(kw, s0 * r0, lp[1]);
            lp[2] = fmaf(kw, s0 * r1, lp[2]); lp[3] = fmaf(kw, r0 * r0, lp[3]);
            lp[4] = fmaf(kw, r0 * r1, lp[4]); lp[5] = fmaf(kw, r1 * r1, lp[5]);
        }
    }
    res[0] = i0; res[1] = i1; res[2] = i2;
#pragma unroll
    for (int ab = 0; ab < 6; ab++) res[3 + ab] = lp[ab];
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

__global__ void __launch_bounds__(MIX_THREADS) k_pass_mix2d(PassArgs a, Rule rule, PassRule pr) {
    extern __shared__ __align__(16) unsigned char s_raw[];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const int nPx = rule.nPx;
    unsigned char *wbase = s_raw + (size_t)wib * mix_warp_bytes(nPx);
    MixWarp &W = *reinterpret_cast<MixWarp *>(wbase);
    float *res = reinterpret_cast<float *>(wbase + ((sizeof(MixWarp) + 15) / 16) * 16);   // [32][nPx][9]
    unsigned short *lst = reinterpret_cast<unsigned short *>(res + 32 * nPx * 9);         // [2][32*nPx]
    const long long gw = (long long)blockIdx.x * MIX_WARPS + wib;
    const long long nw = (long long)gridDim.x * MIX_WARPS;
    unsigned nsub = 0, namb = 0;
    unsigned char mycls[MAXQ];
    for (long long idx = gw; idx < a.count; idx += nw) {
        const int T = a.list[idx];
        int tv[3];
        bool keep[3];
        bool any = false;
#pragma unroll
        for (int r = 0; r < 3; r++) {
            tv[r] = a.T32[(long long)T * 3 + r];
            keep[r] = a.labV[tv[r]] > 0;
            any |= keep[r];
        }
        if (!any || a.labT[T] == 0) continue;
        const ProbParams P = a.probs[a.eprob[T]];
        RowView rows[3];
#pragma unroll
        for (int r = 0; r < 3; r++) {
            rows[r].base = a.rowptr[tv[r]];
            rows[r].n = (int)(a.rowptr[tv[r] + 1] - rows[r].base);
            rows[r].c = a.cols + rows[r].base;
        }
        const double *ET64 = &a.EC[(long long)T * 6];
        const float ohi0 = a.EChi[(long long)T * 6], ohi1 = a.EChi[(long long)T * 6 + 1];
        const float olo0 = a.EClo[(long long)T * 6], olo1 = a.EClo[(long long)T * 6 + 1];
        F2 tl[3];
#pragma unroll
        for (int v = 0; v < 3; v++)
            tl[v] = f2((a.EChi[(long long)T * 6 + 2 * v] - ohi0) + (a.EClo[(long long)T * 6 + 2 * v] - olo0),
                       (a.EChi[(long long)T * 6 + 2 * v + 1] - ohi1) + (a.EClo[(long long)T * 6 + 2 * v + 1] - olo1));
        const float rTT = a.adetf[T];
        DF *vals = (DF *)a.vals;
        for (int k = lane; k < nPx; k += 32) {
            xtoPhys<2>(ET64, &rule.Px[2 * k], &W.x64[2 * k]);
            W.xf[k] = f2((float)(W.x64[2 * k] - ET64[0]), (float)(W.x64[2 * k + 1] - ET64[1]));
        }
        {
            const F2 e1 = tl[1] - tl[0], e2 = tl[2] - tl[0];
            for (int i = lane; i < rule.nPy; i += 32) {
                const float px = rule.Pyf[2 * i], py = rule.Pyf[2 * i + 1];
                W.yT[i] = f2(tl[0].x + e1.x * px + e2.x * py, tl[0].y + e1.y * px + e2.y * py);
            }
        }
        __syncwarp();
        DF D[6];
#pragma unroll
        for (int i = 0; i < 6; i++) D[i] = df_zero();
        const bool frac_close = P.singular && P.close == MTH_FRACTIONAL;
        const float sqf = P.sqdelta_f;
        for (int side = 0; side < 2; side++) {
            const long long lb = side == 0 ? a.out_ptr[T] : a.in_ptr[T];
            const long long le = side == 0 ? a.out_ptr[T + 1] : a.in_ptr[T + 1];
            for (long long p0 = lb; p0 < le; p0 += 32) {
                const long long p = p0 + lane;
                const bool act = p < le;
                const int part = act ? (side == 0 ? a.pB[p] : a.inA[p]) : T;
                int pv[3];
#pragma unroll
                for (int r = 0; r < 3; r++) pv[r] = a.T32[(long long)part * 3 + r];
                bool close = false;
                if (frac_close) {
                    close = (part == T);
#pragma unroll
                    for (int i = 0; i < 3; i++)
#pragma unroll
                        for (int j = 0; j < 3; j++) close |= (tv[i] == pv[j]);
                }
                // owner: partner data and classes
                float pc[6];
#pragma unroll
                for (int j = 0; j < 6; j++)
                    pc[j] = (a.EChi[(long long)part * 6 + j] - ((j & 1) ? ohi1 : ohi0)) + (a.EClo[(long long)part * 6 + j] - ((j & 1) ? olo1 : olo0));
#pragma unroll
                for (int j = 0; j < 6; j++) W.pc[lane][j] = pc[j];
                W.prt[lane] = a.adetf[part];
                W.pid[lane] = part;
                for (int k = 0; k < nPx; k++) {
                    unsigned char c = CLS_OUT;
                    if (act && !close) {
                        F2 Q[3];
                        if (side == 0) {
                            const F2 x = W.xf[k];
                            Q[0] = f2(pc[0] - x.x, pc[1] - x.y); Q[1] = f2(pc[2] - x.x, pc[3] - x.y); Q[2] = f2(pc[4] - x.x, pc[5] - x.y);
                        } else {
                            const float px = rule.Pxf[2 * k], py = rule.Pxf[2 * k + 1];
                            const F2 x = f2(pc[0] + (pc[2] - pc[0]) * px + (pc[4] - pc[0]) * py,
                                            pc[1] + (pc[3] - pc[1]) * px + (pc[5] - pc[1]) * py);
                            Q[0] = tl[0] - x; Q[1] = tl[1] - x; Q[2] = tl[2] - x;
                        }
                        c = (unsigned char)fclassify(Q, sqf);
                    }
                    mycls[k] = c;
                    float *rr = &res[(lane * nPx + k) * 9];
#pragma unroll
                    for (int q = 0; q < 9; q++) rr[q] = 0.f;
                }
                __syncwarp();
                const int nin = build_list(mycls, nPx, CLS_IN, lst);
                const int ncut = build_list(mycls, nPx, CLS_CUT, lst + 32 * nPx);
                // inside items
                for (int c0 = 0; c0 < nin; c0 += 32) {
                    if (c0 + lane < nin) {
                        const int it = lst[c0 + lane];
                        const int k = it >> 5, j = it & 31;
                        float *rr = &res[(j * nPx + k) * 9];
                        if (side == 0) {
                            nsub++;
                            item_out_in(P, rule, pr, W.pc[j], W.prt[j], W.xf[k], rr);
                        } else {
                            const float *q = W.pc[j];
                            const float px = rule.Pxf[2 * k], py = rule.Pxf[2 * k + 1];
                            const F2 x = f2(q[0] + (q[2] - q[0]) * px + (q[4] - q[0]) * py, q[1] + (q[3] - q[1]) * px + (q[5] - q[1]) * py);
                            item_in_in(P, rule, pr, W.yT, rTT, x, rr);
                        }
                    }
                }
                // cut items
                for (int c0 = 0; c0 < ncut; c0 += 32) {
                    if (c0 + lane < ncut) {
                        const int it = lst[32 * nPx + c0 + lane];
                        const int k = it >> 5, j = it & 31;
                        float *rr = &res[(j * nPx + k) * 9];
                        const int pt = W.pid[j];
                        if (side == 0) {
                            item_out_cut(P, rule, W.pc[j], W.xf[k], &W.x64[2 * k], &a.EC[(long long)pt * 6], rr, nsub, namb);
                        } else {
                            const float *q = W.pc[j];
                            const float px = rule.Pxf[2 * k], py = rule.Pxf[2 * k + 1];
                            const F2 x = f2(q[0] + (q[2] - q[0]) * px + (q[4] - q[0]) * py, q[1] + (q[3] - q[1]) * px + (q[5] - q[1]) * py);
                            item_in_cut(P, rule, tl, x, &a.EC[(long long)pt * 6], k, ET64, rr, nsub, namb);
                        }
                    }
                }
                __syncwarp();
                // owner: fold the item sums into the pair's blocks (FP32 quadrature sums, then
                // double-float accumulation of the element block and of the CSR values)
                DF V[9];
#pragma unroll
                for (int i = 0; i < 9; i++) V[i] = df_zero();
                if (act) {
                    if (close) {
                        const long long cs = side == 0 ? close_slot(a.xadj, a.adj, T, part) : close_slot(a.xadj, a.adj, part, T);
                        if (cs < 0) {
                            atomicOr(&a.err[3], 1);
                        } else {
                            const double *cb = &a.closebuf[cs * 36];
                            if (side == 0) {
                                for (int i = 0; i < 3; i++)
                                    for (int j = i; j < 3; j++) D[sym_idx<3>(i, j)] = df_add(D[sym_idx<3>(i, j)], df_from_double(cb[3 * i + j]));
                                for (int i = 0; i < 9; i++) V[i] = df_from_double(cb[9 + i]);
                            } else {
                                for (int i = 0; i < 3; i++)
                                    for (int j = i; j < 3; j++) D[sym_idx<3>(i, j)] = df_add(D[sym_idx<3>(i, j)], df_from_double(cb[18 + 3 * j + i]));
                                for (int i = 0; i < 9; i++) V[i] = df_from_double(cb[27 + i]);
                            }
                        }
                    } else if (side == 0) {
                        float L[6] = {0, 0, 0, 0, 0, 0}, N[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
                        for (int k = 0; k < nPx; k++) {
                            const float *rr = &res[(lane * nPx + k) * 9];
#pragma unroll
                            for (int ab = 0; ab < 6; ab++) L[ab] = fmaf(pr.cxx[6 * k + ab], rr[0], L[ab]);
#pragma unroll
                            for (int r = 0; r < 3; r++) {
                                const float c = pr.cx[3 * k + r];
                                N[3 * r + 0] = fmaf(c, rr[1], N[3 * r + 0]);
                                N[3 * r + 1] = fmaf(c, rr[2], N[3 * r + 1]);
                                N[3 * r + 2] = fmaf(c, rr[3], N[3 * r + 2]);
                            }
                        }
#pragma unroll
                        for (int i = 0; i < 6; i++) D[i] = df_add(D[i], L[i] * rTT);
#pragma unroll
                        for (int i = 0; i < 9; i++) V[i] = DF{N[i] * rTT, 0.f};
                    } else {
                        float LP[6] = {0, 0, 0, 0, 0, 0}, NP[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
                        for (int k = 0; k < nPx; k++) {
                            const float *rr = &res[(lane * nPx + k) * 9];
                            const float dk = pr.dxf[k];
#pragma unroll
                            for (int ab = 0; ab < 6; ab++) LP[ab] = fmaf(dk, rr[3 + ab], LP[ab]);
#pragma unroll
                            for (int r = 0; r < 3; r++) {
                                const float c = pr.cx[3 * k + r];
                                NP[3 * r + 0] = fmaf(c, rr[0], NP[3 * r + 0]);
                                NP[3 * r + 1] = fmaf(c, rr[1], NP[3 * r + 1]);
                                NP[3 * r + 2] = fmaf(c, rr[2], NP[3 * r + 2]);
                            }
                        }
                        const float adetA = W.prt[lane];
#pragma unroll
                        for (int i = 0; i < 6; i++) D[i] = df_add(D[i], LP[i] * adetA);
#pragma unroll
                        for (int i = 0; i < 9; i++) V[i] = DF{NP[i] * adetA, 0.f};
                    }
                }
                // scatter: out side termNonloc[r][b] -> A[T[r], bT[b]]; in side
                // termNonlocPrime[c][r] -> A[T[r], aT[c]] (both with the minus sign)
#pragma unroll
                for (int c = 0; c < 3; c++) {
                    DF v[3];
#pragma unroll
                    for (int r = 0; r < 3; r++) {
                        const DF t = side == 0 ? V[3 * r + c] : V[3 * c + r];
                        v[r] = DF{-t.hi, -t.lo};
                    }
                    warp_scatter_df<3>(act ? pv[c] : -1, v, rows, keep, vals, &a.err[3], a.touched);
                }
                __syncwarp();
            }
        }
#pragma unroll
        for (int i = 0; i < 6; i++) D[i] = warp_sum_df(D[i]);
        if (lane == 0) {
            for (int r = 0; r < 3; r++) {
                if (!keep[r]) continue;
                for (int c = 0; c < 3; c++) {
                    const long long slot = rv_find(rows[r], tv[c]);
                    if (slot < 0) { atomicOr(&a.err[3], 1); continue; }
                    vals[slot] = df_add(vals[slot], D[r <= c ? sym_idx<3>(r, c) : sym_idx<3>(c, r)]);
                    if (a.touched) a.touched[slot] = 1;
                }
            }
        }
        __syncwarp();
    }
    nsub = warp_sum(nsub);
    namb = warp_sum(namb);
    if (lane == 0) {
        if (nsub && a.n_subtri) atomicAdd(a.n_subtri, (unsigned long long)nsub);
        if (namb && a.n_amb) atomicAdd(a.n_amb, (unsigned long long)namb);
    }
}

}  // namespace nlg
