// Mixed-precision barycenter pass (integrate_baryCenter, integration.cpp:910-1018, with
// method_baryCenter, :1262-1280): one-sided, work-compacted, fixed-point scatter, 2D and 3D.
//
// The rule has no Prime blocks: a pair (T, b) adds 2 |T| psi_a psi_b dx innerLocal into A[T, T]
// and -2 |T| psi_a dx innerNonloc into A[T, b], where an outer point x_k of T counts when the
// ball around it contains b's barycenter. So each element writes only its own rows; with the
// contributions added as 64-bit fixed-point integers (slots.cuh) no coloring is needed, and one
// persistent launch takes elements from a global counter.
//
// Per batch of 32 pairs, the owner lane tests its pair's outer points (FP32 distance with a
// certified margin, exact FP64 test inside the margin), the (pair, point) items whose ball
// contains the barycenter are compacted and integrated 32 at a time over the full inner element,
// and the owner lane folds them in a fixed order. Only off-diagonal entries are accumulated; the
// matrix rows sum to zero, and k_row_diag sets the diagonal entries from the row sums. Lanes sharing
// a partner vertex add their integers; all lanes then share the slot lookups in T's rows.
#pragma once
#include "passes_mix.cuh"

namespace nlg {

constexpr int BARY_WARPS = 4;
constexpr int BARY_THREADS = 32 * BARY_WARPS;

template <int DIM>
struct BaryWarp {
    double x64[MAXQ * DIM];             // outer points of T (FP64, exact)
    float xf[MAXQ * DIM];               // outer points of T, local (relative to T's vertex 0)
    float pc[32][DIM * (DIM + 1)];      // partner element, local coordinates
    float prt[32];                      // partner |det|
    long long rhb[DIM + 1], rrb[DIM + 1];   // T's rows: hash table start, CSR row start
    unsigned rmask[DIM + 1];            // T's rows: slot map size field (0xffffffff: no row), see RowHash
    int rlo[DIM + 1];                   // T's rows: first window word (window-rank map)
    int tvs[DIM + 1];                   // T's vertices
};
template <int DIM>
struct BaryEntry {   // one partner vertex of a batch and its integer sums over T's rows
    int col, pad;
    long long v[DIM + 1];
};
template <int DIM>
__host__ __device__ constexpr size_t bary_res_bytes(int nPx) {
    return (size_t)32 * nPx * (DIM + 2) * 4 > (size_t)32 * (DIM + 1) * sizeof(BaryEntry<DIM>)
               ? (size_t)32 * nPx * (DIM + 2) * 4
               : (size_t)32 * (DIM + 1) * sizeof(BaryEntry<DIM>);
}
template <int DIM>
__host__ __device__ constexpr size_t bary_warp_bytes(int nPx) {
    // BaryWarp + item results [32][nPx][DIM+2] (or the scatter list) + inside list [32*nPx] shorts
    return ((sizeof(BaryWarp<DIM>) + 15) / 16) * 16 + bary_res_bytes<DIM>(nPx) + (size_t)32 * nPx * 2 + 16;
}

// Kernel value from r^2 = |x - y|^2 (model.cpp:25-28, 52-60, 62-65, 126-138), FP32.
__device__ __forceinline__ float kernel_f32_r2(const ProbParams &P, float r2) {
    switch (P.kernel) {
    case KER_PARABOLA: return P.kc_f * (P.sqdelta_f - r2);
    case KER_FRACTIONAL: return P.kc_f * exp2f(-0.5f * P.expo_f * log2f(r2));
    default: return P.kc_f;
    }
}

// CK: the launch covers constant-kernel problems only; an item's sums over the full inner element
// are then kc |b| times the rule's precomputed element sums.
template <int DIM, bool CK>
__global__ void __launch_bounds__(BARY_THREADS) k_pass_bary(MixArgs ma, Rule rule, PassRule pr) {
    constexpr int dV = DIM + 1, NS = dV * (dV + 1) / 2, RN = DIM + 2;
    extern __shared__ __align__(16) unsigned char s_raw[];
    const PassArgs &a = ma.p;
    const SlotMap &sm = ma.m;
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const int nPx = rule.nPx;
    unsigned char *wbase = s_raw + (size_t)wib * bary_warp_bytes<DIM>(nPx);
    BaryWarp<DIM> &W = *reinterpret_cast<BaryWarp<DIM> *>(wbase);
    float *res = reinterpret_cast<float *>(wbase + ((sizeof(BaryWarp<DIM>) + 15) / 16) * 16);   // [32][nPx][RN]
    unsigned short *lst = reinterpret_cast<unsigned short *>(reinterpret_cast<unsigned char *>(res) + bary_res_bytes<DIM>(nPx));
    BaryEntry<DIM> *slist = reinterpret_cast<BaryEntry<DIM> *>(res);
    long long *vals = reinterpret_cast<long long *>(a.vals);
    int *ovf = &a.err[5];
    bool bad = false;   // a contribution outside the fixed-point range (reported at the end)
    bool miss = false;  // a matrix slot not found (reported at the end)
    unsigned nsub = 0, namb = 0, nitin = 0;
    unsigned char mycls[MAXQ];
    for (;;) {
        int idx = 0;
        if (lane == 0) idx = atomicAdd(ma.work, 1);
        idx = __shfl_sync(FULL, idx, 0);
        if (idx >= a.count) break;
        const int T = a.list ? a.list[idx] : idx;
        const long long lb = a.out_ptr[T], le = a.out_cnt ? lb + a.out_cnt[T] : a.out_ptr[T + 1];
        if (lb == le || a.labT[T] == 0) continue;
        int tv[dV];
        unsigned keepmask = 0;
#pragma unroll
        for (int r = 0; r < dV; r++) {
            tv[r] = a.T32[(long long)T * dV + r];
            if (a.labV[tv[r]] > 0) keepmask |= 1u << r;
        }
        if (lane < dV) {
            RowHash h;
            h.hb = h.rb = 0;
            h.mask = 0xffffffffu;
            h.lo = 0;
            if (keepmask & (1u << lane)) h = row_hash(sm, a.T32[(long long)T * dV + lane]);
            W.rhb[lane] = h.hb;
            W.rrb[lane] = h.rb;
            W.rmask[lane] = h.mask;
            W.rlo[lane] = h.lo;
            W.tvs[lane] = a.T32[(long long)T * dV + lane];
        }
        const ProbParams P = a.probs[a.eprob[T]];
        const double *ET64 = &a.EC[(long long)T * DIM * dV];
        float ohi[DIM], olo[DIM];
#pragma unroll
        for (int j = 0; j < DIM; j++) {
            ohi[j] = a.EChi[(long long)T * DIM * dV + j];
            olo[j] = a.EClo[(long long)T * DIM * dV + j];
        }
        const float rTT = a.adetf[T];
        for (int k = lane; k < nPx; k += 32) {
            xtoPhys<DIM>(ET64, &rule.Px[DIM * k], &W.x64[DIM * k]);
#pragma unroll
            for (int j = 0; j < DIM; j++) W.xf[DIM * k + j] = (float)(W.x64[DIM * k + j] - ET64[j]);
        }
        __syncwarp();
        long long D[NS];   // termLocal of T's pairs, integer sums
#pragma unroll
        for (int i = 0; i < NS; i++) D[i] = 0;
        const float sqlo = P.sqdelta_f * (1.f - MARG_D), sqhi = P.sqdelta_f * (1.f + MARG_D);
        int part_next = lb + lane < le ? a.pB[lb + lane] : T;   // partners one batch ahead
        for (long long p0 = lb; p0 < le; p0 += 32) {
            const long long p = p0 + lane;
            const bool act = p < le;
            const int part = part_next;
            part_next = p + 32 < le ? a.pB[p + 32] : T;
            if (!CK) {   // the inner quadrature needs the partner's vertices
#pragma unroll
                for (int j = 0; j < DIM * dV; j++)
                    W.pc[lane][j] = (a.EChi[(long long)part * DIM * dV + j] - ohi[j % DIM]) +
                                    (a.EClo[(long long)part * DIM * dV + j] - olo[j % DIM]);
            }
            W.prt[lane] = a.adetf[part];
            float bf[DIM];
            bary_offset<DIM>(a.BCf, part, ohi, olo, bf);
            // owner: which outer points see the partner's barycenter inside the ball
            bool have_b64 = false;
            double b64[DIM];
            float inv[RN];   // constant kernel: an item's sums
            unsigned inm = 0;   // constant kernel: outer points whose ball holds the barycenter
            if (CK) {
                const float kr = P.kc_f * W.prt[lane];
#pragma unroll
                for (int q = 0; q < RN; q++) inv[q] = kr * pr.insum[q];
            }
            for (int k = 0; k < nPx; k++) {
                unsigned char c = 0;
                if (act) {
                    float d2 = 0.f;
#pragma unroll
                    for (int j = 0; j < DIM; j++) {
                        const float d = W.xf[DIM * k + j] - bf[j];
                        d2 = fmaf(d, d, d2);
                    }
                    if (d2 < sqlo) c = 1;
                    else if (d2 <= sqhi) {   // inside the margin: the exact test decides
                        namb++;
                        if (!have_b64) { xbary<DIM>(&a.EC[(long long)part * DIM * dV], b64); have_b64 = true; }
                        c = xbaryInside<DIM>(&W.x64[DIM * k], b64, P.sqdelta) ? 1 : 0;
                    }
                }
                nitin += c;
                if (CK) {
                    inm |= (unsigned)c << k;
                    nsub += c;
                } else {
                    mycls[k] = c;
                    float *rr = &res[(lane * nPx + k) * RN];
#pragma unroll
                    for (int q = 0; q < RN; q++) rr[q] = 0.f;
                }
            }
            __syncwarp();
            const int nin = CK ? 0 : build_list(mycls, nPx, 1, lst);
            for (int c0 = 0; c0 < nin; c0 += 32) {
                if (c0 + lane < nin) {
                    const int it = lst[c0 + lane];
                    const int k = it >> 5, j = it & 31;
                    nsub++;
                    const float *q = W.pc[j];
                    const float rb = W.prt[j];
                    float e[DIM][DIM], b0[DIM];   // y - x = b0 + sum_c e[c] P_c
#pragma unroll
                    for (int d = 0; d < DIM; d++) {
                        b0[d] = q[d] - W.xf[DIM * k + d];
#pragma unroll
                        for (int c = 0; c < DIM; c++) e[c][d] = q[DIM * (c + 1) + d] - q[d];
                    }
                    float iL = 0.f, iN[dV];
#pragma unroll
                    for (int t = 0; t < dV; t++) iN[t] = 0.f;
                    for (int i = 0; i < rule.nPy; i++) {
                        float r2 = 0.f;
#pragma unroll
                        for (int d = 0; d < DIM; d++) {
                            float z = b0[d];
#pragma unroll
                            for (int c = 0; c < DIM; c++) z = fmaf(e[c][d], pr.pyf[DIM * i + c], z);
                            r2 = fmaf(z, z, r2);
                        }
                        const float kw = kernel_f32_r2(P, r2) * rb;
                        iL = fmaf(kw, rule.dyf[i], iL);
#pragma unroll
                        for (int t = 0; t < dV; t++) iN[t] = fmaf(kw, pr.cy[dV * i + t], iN[t]);
                    }
                    float *rr = &res[(j * nPx + k) * RN];
                    rr[0] = iL;
#pragma unroll
                    for (int t = 0; t < dV; t++) rr[1 + t] = iN[t];
                }
            }
            __syncwarp();
            // owner: fold, weight 2 (integration.cpp:1001-1013), fixed point from here on
            long long nx[dV * dV];
#pragma unroll
            for (int i = 0; i < dV * dV; i++) nx[i] = 0;
            if (act) {
                float L[NS], N[dV * dV];
#pragma unroll
                for (int i = 0; i < NS; i++) L[i] = 0.f;
#pragma unroll
                for (int i = 0; i < dV * dV; i++) N[i] = 0.f;
                if (CK) {   // every item's sums are inv: the folds are inv times the mask's rule sums
                    float sx[NS], cxs[dV];
                    if (inm == (nPx == 32 ? 0xffffffffu : (1u << nPx) - 1u)) {
#pragma unroll
                        for (int i = 0; i < NS; i++) sx[i] = pr.xsum[i];
#pragma unroll
                        for (int r = 0; r < dV; r++) cxs[r] = pr.xsum[NS + r];
                    } else {
#pragma unroll
                        for (int i = 0; i < NS; i++) sx[i] = 0.f;
#pragma unroll
                        for (int r = 0; r < dV; r++) cxs[r] = 0.f;
                        for (unsigned mm = inm; mm; mm &= mm - 1) {
                            const int k = __ffs(mm) - 1;
#pragma unroll
                            for (int i = 0; i < NS; i++) sx[i] += pr.cxx[NS * k + i];
#pragma unroll
                            for (int r = 0; r < dV; r++) cxs[r] += pr.cx[dV * k + r];
                        }
                    }
#pragma unroll
                    for (int i = 0; i < NS; i++) L[i] = sx[i] * inv[0];
#pragma unroll
                    for (int r = 0; r < dV; r++)
#pragma unroll
                        for (int t = 0; t < dV; t++) N[dV * r + t] = cxs[r] * inv[1 + t];
                }
                for (int k = 0; k < (CK ? 0 : nPx); k++) {
                    const float *rr = &res[(lane * nPx + k) * RN];
#pragma unroll
                    for (int s = 0; s < NS; s++) L[s] = fmaf(pr.cxx[NS * k + s], rr[0], L[s]);
#pragma unroll
                    for (int r = 0; r < dV; r++) {
                        const float c = pr.cx[dV * k + r];
#pragma unroll
                        for (int t = 0; t < dV; t++) N[dV * r + t] = fmaf(c, rr[1 + t], N[dV * r + t]);
                    }
                }
                // off-diagonal entries only: every kept row sums to zero (each pair's blocks do),
                // so k_row_diag sets each diagonal entry to minus its row's other entries, the same
                // integer a per-pair balance of the block diagonals would give
#pragma unroll
                for (int r = 0; r < dV; r++)
#pragma unroll
                    for (int c = r + 1; c < dV; c++) {
                        const int i = sym_idx<dV>(r, c);
                        D[i] += fx64(2.f * L[i] * rTT, P.fx_mul, bad);
                    }
#pragma unroll
                for (int i = 0; i < dV * dV; i++) nx[i] = fx64(2.f * N[i] * rTT, P.fx_mul, bad);
            }
            // termNonloc into A[T, b] (minus sign): group sums per partner vertex, shared lookups
            __syncwarp();
            int nent = 0;
#pragma unroll 1
            for (int c = 0; c < dV; c++) {
                int col = -1;
                if (act) {
#pragma unroll
                    for (int t = 0; t < dV; t++)
                        if (t == c) col = a.T32[(long long)part * dV + t];
                }
                const unsigned grp = __match_any_sync(FULL, col);
                const bool leader = (__ffs(grp) - 1) == lane;
                const int maxn = __reduce_max_sync(FULL, (unsigned)__popc(grp));
                long long own[dV], sn[dV];
#pragma unroll
                for (int r = 0; r < dV; r++) {
                    long long v = 0;
#pragma unroll
                    for (int t = 0; t < dV; t++)
                        if (t == c) v = nx[dV * r + t];
                    own[r] = sn[r] = v;
                }
                unsigned rest = grp & ~(1u << lane);
                for (int it = 1; it < maxn; it++) {
                    const int src = rest ? __ffs(rest) - 1 : lane;
                    const bool use = rest != 0;
                    if (rest) rest &= rest - 1;
#pragma unroll
                    for (int r = 0; r < dV; r++) {
                        const long long t = shfl64(own[r], src);
                        if (use) sn[r] += t;
                    }
                }
                const bool put = leader && col >= 0;
                const unsigned m = __ballot_sync(FULL, put);
                if (put) {
                    BaryEntry<DIM> &e = slist[nent + __popc(m & lanemask_lt())];
                    e.col = col;
#pragma unroll
                    for (int r = 0; r < dV; r++) e.v[r] = sn[r];
                }
                nent += __popc(m);
            }
            __syncwarp();
            for (int w = lane; w < dV * nent; w += 32) {
                const int e = w / dV, r = w - dV * e;
                RowHash h;
                h.hb = W.rhb[r]; h.rb = W.rrb[r]; h.mask = W.rmask[r]; h.lo = W.rlo[r];
                if (h.mask == 0xffffffffu) continue;   // T's vertex r has no row
                if (slist[e].col == W.tvs[r]) continue;   // the matrix diagonal: from the row sum
                const long long s = slot_find_row(sm, h, slist[e].col);
                if (s < 0) miss = true;
                else red_add(vals, s, -slist[e].v[r]);
            }
            __syncwarp();
        }
        // termLocal of all of T's pairs into T's diagonal block
#pragma unroll
        for (int i = 0; i < NS; i++)
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) D[i] += (long long)__shfl_xor_sync(FULL, (unsigned long long)D[i], o);
        if (lane < dV * dV && lane / dV != lane % dV) {   // off-diagonal entries of T's block
            const int r = lane / dV, c = lane % dV;
            RowHash h;
            h.hb = W.rhb[r]; h.rb = W.rrb[r]; h.mask = W.rmask[r]; h.lo = W.rlo[r];
            if (h.mask != 0xffffffffu) {
                long long d = 0;
                const int si = r <= c ? sym_idx<dV>(r, c) : sym_idx<dV>(c, r);
#pragma unroll
                for (int i = 0; i < NS; i++)
                    if (i == si) d = D[i];
                const long long s = slot_find_row(sm, h, a.T32[(long long)T * dV + c]);
                if (s < 0) miss = true;
                else red_add(vals, s, d);
            }
        }
        __syncwarp();
    }
    if (__any_sync(FULL, bad) && lane == 0) atomicOr(ovf, 1);
    if (__any_sync(FULL, miss) && lane == 0) atomicOr(&a.err[3], 1);
    nsub = warp_sum(nsub);
    namb = warp_sum(namb);
    nitin = warp_sum(nitin);
    if (lane == 0) {
        if (nsub && a.n_subtri) atomicAdd(a.n_subtri, (unsigned long long)nsub);
        if (namb && a.n_amb) atomicAdd(a.n_amb, (unsigned long long)namb);
        if (nitin && a.n_in) atomicAdd(a.n_in, (unsigned long long)nitin);
    }
}

// Completion of the barycenter pass: each row's diagonal entry becomes minus the sum of its other
// entries (the pass left it out; every kept row sums to zero, rows the pass did not write stay
// zero). One warp per row.
__global__ void k_row_diag(const long long *__restrict__ rowptr, const int *__restrict__ cols, long long nrows,
                           long long *__restrict__ vals) {
    const int lane = threadIdx.x & 31;
    const long long gw = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const long long nw = ((long long)gridDim.x * blockDim.x) >> 5;
    for (long long t = gw; t < nrows; t += nw) {
        const long long b = rowptr[t], e = rowptr[t + 1];
        long long off = 0, dslot = -1;
        for (long long s = b + lane; s < e; s += 32) {
            if (cols[s] == (int)t) dslot = s;
            else off += vals[s];
        }
        off = (long long)warp_sum((unsigned long long)off);
        if (dslot >= 0) vals[dslot] = -off;
    }
}

}  // namespace nlg
