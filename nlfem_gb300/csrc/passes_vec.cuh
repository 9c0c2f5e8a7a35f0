// Vector-valued kernels (outdim OD > 1): the FP64 pair quadrature with the reference's general
// block indexing, and the load vector of vector forcings.
//
// One thread per ordered pair (aT, bT) of the search's pair list computes the pair's four blocks
// of size (dV OD)^2 in FP64 with the reference's loops:
//   retriangulate  integrate_retriangulate (integration.cpp:345-540): kernel matrices k(x, y) and
//                  k(y, x), the inner sums innerLocal[OD^2], innerNonloc[dV OD^2], ... folded as
//                  termLocal[dV OD a + b] += |aT| psi(a / OD) psi(b / OD) dx innerLocal[OD (a % OD) + b % OD]
//   baryCenter     integrate_baryCenter (integration.cpp:910-1018), weight 2, no prime blocks
//   fractional     integrate_fractional (integration.cpp:187-288) on the Duffy points, the kernel
//                  matrix entry of (aOut, bOut) times psixy[a] psixy[b]
//   weakSingular   integrate_weakSingular (integration.cpp:82-185)
// and adds them to the expanded matrix (Cassemble.cpp:721-770):
//   A[OD aV[a/OD] + a%OD, OD aV[b/OD] + b%OD] += termLocal,  A[.., OD bV[b/OD] + b%OD] -= termNonloc
//   (rows of aT's vertices with label > 0),
//   A[OD bV[b/OD] + b%OD, OD bV[a/OD] + a%OD] += termLocalPrime,  A[.., OD aV[a/OD] + a%OD] -= termNonlocPrime
//   (rows of bT's vertices with label > 0).
// The expanded pattern is the vertex pattern with every entry an OD x OD tile: row OD v + i holds
// the columns OD w + j of the vertex row v, in order, at slot OD^2 rowptr[v] + i OD n_v + OD pos + j
// (pos the place of w in row v, n_v its length). Values are 128-bit fixed-point sums of the FP64
// contributions (order-independent, so deterministic); the finish drops exact zeros.
#pragma once
#include "quadrature.cuh"

namespace nlg {

struct VecArgs {
    const int *pA, *pB, *T32, *labV, *labT, *eprob;
    const double *EC, *adet;
    const ProbParams *probs;
    const long long *rowptr;
    const int *cols;
    unsigned long long *acc;   // 2 words per expanded slot
    unsigned *tiny;
    long long P;
    int *err;                  // [3] slot not found, [4] singular toRef
    unsigned long long *n_close, *n_subtri;
};

template <int OD>
__device__ __forceinline__ void vec_add(const VecArgs &a, const ProbParams &P, int v, int i, int w, int j, double val) {
    if (val == 0.0) return;   // adds nothing; the slot exists in the pattern either way
    const long long s = find_slot(a.rowptr, a.cols, v, w);
    if (s < 0) { atomicOr(&a.err[3], 1); return; }
    const long long rb = a.rowptr[v], n = a.rowptr[v + 1] - rb;
    const long long idx = (long long)OD * OD * rb + (long long)i * OD * n + (long long)OD * (s - rb) + j;
    fx_atomic_add(&a.acc[2 * idx], val, P.scale_exp, &a.tiny[idx]);
}

// Block index of the four (dV OD)^2 blocks
template <int DIM, int OD>
struct VB {
    static constexpr int dV = DIM + 1, NB = dV * OD, NN = NB * NB;
};

// integrate_retriangulate with the general outdim indexing (2D).
template <int OD>
__device__ int vec_retriangulate(const ProbParams &P, const Rule &rule, const double *Ea, const double *Eb,
                                 double adet_a, double *L, double *N, double *LP, double *NP, int *err, int &nsub) {
    constexpr int dV = 3, O2 = OD * OD, NB = dV * OD;
    double R[18];
    int interacts = 0;
    for (int k = 0; k < rule.nPx; k++) {
        double x[2];
        xtoPhys<2>(Ea, &rule.Px[2 * k], x);
        const int Rdx = xretriangulate(x, Eb, P.sqdelta, P.caps, R);
        interacts |= (Rdx >= 3);
        nsub += Rdx >= 3 ? Rdx - 2 : 0;
        double iL[O2], iN[O2 * dV], iNP[O2 * dV];
#pragma unroll
        for (int o = 0; o < O2; o++) iL[o] = 0;
#pragma unroll
        for (int o = 0; o < O2 * dV; o++) { iN[o] = 0; iNP[o] = 0; }
        for (int r = 0; r + 2 < Rdx; r++) {
            const double tri[6] = {R[0], R[1], R[2 * r + 2], R[2 * r + 3], R[2 * r + 4], R[2 * r + 5]};
            const double rTdet = xabsDet2(tri);
            for (int i = 0; i < rule.nPy; i++) {
                double y[2];
                y[0] = (tri[2] - tri[0]) * rule.Py[2 * i] + (tri[4] - tri[0]) * rule.Py[2 * i + 1] + tri[0];
                y[1] = (tri[3] - tri[1]) * rule.Py[2 * i] + (tri[5] - tri[1]) * rule.Py[2 * i + 1] + tri[1];
                double kv[O2], kp[O2];
                kernel_field_f64<OD>(P, x, y, kv);
                kernel_field_f64<OD>(P, y, x, kp);
                const double w = rule.dy[i] * rTdet;
#pragma unroll
                for (int o = 0; o < O2; o++) iL[o] += kv[o] * w;
                double ref[2];
                if (!xtoRef(Eb, y, ref)) atomicOr(&err[4], 1);
                const double psi[3] = {1.0 - ref[0] - ref[1], ref[0], ref[1]};
#pragma unroll
                for (int b = 0; b < dV * O2; b++) {
                    iN[b] += psi[b / O2] * kv[b % O2] * w;
                    iNP[b] += psi[b / O2] * kp[b % O2] * w;
                }
                const double wl = w * rule.dx[k] * adet_a;
                for (int aa = 0; aa < dV; aa++)
                    for (int b = 0; b < dV; b++)
#pragma unroll
                        for (int o = 0; o < O2; o++)
                            LP[aa * O2 * dV + (o / OD) * OD * dV + b * OD + o % OD] += psi[aa] * psi[b] * kp[o] * wl;
            }
        }
        const double wx = adet_a * rule.dx[k];
        for (int aa = 0; aa < NB; aa++) {
            const double pa = rule.psix[3 * k + aa / OD] * wx;
            for (int b = 0; b < NB; b++) {
                L[NB * aa + b] += pa * rule.psix[3 * k + b / OD] * iL[OD * (aa % OD) + b % OD];
                const int q = (aa % OD) * OD + O2 * (b / OD) + b % OD;
                N[NB * aa + b] += pa * iN[q];
                NP[NB * aa + b] += pa * iNP[q];
            }
        }
    }
    return interacts | P.full_search;
}

// integrate_baryCenter with the general outdim indexing (2D or 3D): weight 2, no prime blocks.
template <int DIM, int OD>
__device__ int vec_barycenter(const ProbParams &P, const Rule &rule, const double *Ea, const double *Eb,
                              double adet_a, double adet_b, double *L, double *N, int &nsub) {
    constexpr int dV = DIM + 1, O2 = OD * OD, NB = dV * OD;
    double bc[DIM];
    xbary<DIM>(Eb, bc);
    int interacts = 0;
    for (int k = 0; k < rule.nPx; k++) {
        double x[DIM];
        xtoPhys<DIM>(Ea, &rule.Px[DIM * k], x);
        if (!xbaryInside<DIM>(x, bc, P.sqdelta)) continue;
        interacts = 1;
        nsub++;
        double iL[O2], iN[O2 * dV];
#pragma unroll
        for (int o = 0; o < O2; o++) iL[o] = 0;
#pragma unroll
        for (int o = 0; o < O2 * dV; o++) iN[o] = 0;
        for (int i = 0; i < rule.nPy; i++) {
            double y[DIM];
            xtoPhys<DIM>(Eb, &rule.Py[DIM * i], y);
            double kv[O2];
            kernel_field_f64<OD>(P, x, y, kv);
#pragma unroll
            for (int o = 0; o < O2; o++) iL[o] += adet_b * kv[o] * rule.dy[i];
            kernel_field_f64<OD>(P, y, x, kv);
#pragma unroll
            for (int b = 0; b < dV * O2; b++) iN[b] += rule.psiy[dV * i + b / O2] * kv[b % O2] * rule.dy[i] * adet_b;
        }
        for (int aa = 0; aa < NB; aa++) {
            const double pa = 2 * adet_a * rule.psix[dV * k + aa / OD];
            for (int b = 0; b < NB; b++) {
                L[NB * aa + b] += pa * rule.psix[dV * k + b / OD] * rule.dx[k] * iL[OD * (aa % OD) + b % OD];
                N[NB * aa + b] += pa * rule.dx[k] * iN[(aa % OD) * OD + O2 * (b / OD) + b % OD];
            }
        }
    }
    return interacts | P.full_search;
}

// integrate_fractional / integrate_weakSingular with join() (integration.cpp:82-288, 1913-1958),
// general outdim indexing, FP64, in one thread.
template <int OD>
__device__ void vec_close(const ProbParams &P, const Duffy &d, const int *aV, const int *bV, const double *Ea,
                          const double *Eb, double *L, double *N, double *LP, double *NP) {
    constexpr int dV = 3, NB = dV * OD;
    int nEqual = 0, AinB[3] = {0, 0, 0}, BinA[3] = {0, 0, 0}, argA[3], argB[3];
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++)
            if (aV[i] == bV[j]) {
                AinB[i] += 1; BinA[j] += 1;
                argA[nEqual] = i; argB[nEqual] = j;
                nEqual++;
            }
    int ia = 0, ib = 0;
    for (int i = 0; i < 3; i++) {
        if (!AinB[i]) { argA[nEqual + ia] = i; ia++; }
        if (!BinA[i]) { argB[nEqual + ib] = i; ib++; }
    }
    if (nEqual < 1 || nEqual > 3) return;
    double EA[6], EB[6];
    for (int k = 0; k < 3; k++) {
        EA[2 * k] = Ea[2 * argA[k]]; EA[2 * k + 1] = Ea[2 * argA[k] + 1];
        EB[2 * k] = Eb[2 * argB[k]]; EB[2 * k + 1] = Eb[2 * argB[k] + 1];
    }
    const double dA = xabsDet2(EA), dB = xabsDet2(EB);
    const int c = nEqual - 1;
    const int nT = nEqual == 1 ? 2 : (nEqual == 2 ? 5 : 6);
    const bool weak = P.close == MTH_WEAKSING;
    const int nL = 2 * dV - nEqual, shift = dV - nEqual;
    for (int idx = 0; idx < nT * d.nPg; idx++) {
        const int k = idx % d.nPg;
        const double *ac = &d.alpha[c][(long long)idx * 4];   // xi factored out
        double x[2], y[2];
        x[0] = (EA[2] - EA[0]) * ac[0] + (EA[4] - EA[0]) * ac[1] + EA[0];
        x[1] = (EA[3] - EA[1]) * ac[0] + (EA[5] - EA[1]) * ac[1] + EA[1];
        y[0] = (EB[2] - EB[0]) * ac[2] + (EB[4] - EB[0]) * ac[3] + EB[0];
        y[1] = (EB[3] - EB[1]) * ac[2] + (EB[5] - EB[1]) * ac[3] + EB[1];
        double kv[OD * OD];
        kernel_field_f64<OD>(P, x, y, kv);
        if (weak) {   // basis at the points with xi kept, weight xi^(1 - 2s)
            const double *au = &d.alphaU[c][(long long)idx * 4];
            const double px[3] = {1.0 - au[0] - au[1], au[0], au[1]};
            const double py[3] = {1.0 - au[2] - au[3], au[2], au[3]};
            const double base = d.tdetW[c][idx] * d.dg[k] * dA * dB;
            for (int a = 0; a < dV; a++)
                for (int ao = 0; ao < OD; ao++)
                    for (int b = 0; b < dV; b++)
                        for (int bo = 0; bo < OD; bo++) {
                            const double f = kv[OD * ao + bo] * base;
                            L[NB * (argA[a] * OD + ao) + argA[b] * OD + bo] += f * px[a] * px[b];
                            LP[NB * (argB[a] * OD + ao) + argB[b] * OD + bo] += f * py[a] * py[b];
                            N[NB * (argA[a] * OD + ao) + argB[b] * OD + bo] += f * px[a] * py[b];
                            NP[NB * (argA[a] * OD + ao) + argB[b] * OD + bo] += f * px[a] * py[b];
                        }
        } else {
            const double px[3] = {1.0 - ac[0] - ac[1], ac[0], ac[1]};
            const double py[3] = {1.0 - ac[2] - ac[3], ac[2], ac[3]};
            double pxy[6];
            for (int a = 0; a < nEqual; a++) pxy[a] = px[a] - py[a];
            for (int a = nEqual; a < dV; a++) {
                pxy[a] = px[a];
                pxy[a + shift] = -py[a];
            }
            const double base = d.tdet[c][idx] * d.dg[k] * dA * dB;
            for (int a = 0; a < nL; a++)
                for (int ao = 0; ao < OD; ao++)
                    for (int b = 0; b < nL; b++)
                        for (int bo = 0; bo < OD; bo++) {
                            const double f = kv[OD * ao + bo] * base * pxy[a] * pxy[b];
                            if (a < dV) {
                                if (b < dV) L[NB * (argA[a] * OD + ao) + argA[b] * OD + bo] += f;
                                else N[NB * (argA[a] * OD + ao) + argB[b - shift] * OD + bo] -= f;
                            } else {
                                if (b < dV) NP[NB * (argA[b] * OD + ao) + argB[a - shift] * OD + bo] -= f;
                                else LP[NB * (argB[a - shift] * OD + ao) + argB[b - shift] * OD + bo] += f;
                            }
                        }
        }
    }
}

// One thread per ordered pair: the four blocks, then the scatter.
template <int DIM, int OD>
__global__ void __launch_bounds__(128) k_quad_vec(VecArgs a, Rule rule, Duffy d) {
    constexpr int dV = DIM + 1, NB = dV * OD, NN = NB * NB;
    const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    int nsub = 0;
    bool close = false;
    if (p < a.P) {
        const int aT = a.pA[p], bT = a.pB[p];
        const ProbParams P = a.probs[a.eprob[aT]];
        int aV[dV], bV[dV];
#pragma unroll
        for (int i = 0; i < dV; i++) { aV[i] = a.T32[(long long)aT * dV + i]; bV[i] = a.T32[(long long)bT * dV + i]; }
        close = P.singular && share_vertex(aV, bV, dV);
        const int method = close ? P.close : P.remote;
        double Ea[DIM * dV], Eb[DIM * dV];
#pragma unroll
        for (int i = 0; i < DIM * dV; i++) { Ea[i] = a.EC[(long long)aT * DIM * dV + i]; Eb[i] = a.EC[(long long)bT * DIM * dV + i]; }
        double L[NN], N[NN], LP[NN], NP[NN];
        for (int i = 0; i < NN; i++) { L[i] = 0; N[i] = 0; LP[i] = 0; NP[i] = 0; }
        bool prime = true;
        if (DIM == 2 && (method == MTH_FRACTIONAL || method == MTH_WEAKSING)) {
            vec_close<OD>(P, d, aV, bV, Ea, Eb, L, N, LP, NP);
        } else if (method == MTH_BARYCENTER) {
            vec_barycenter<DIM, OD>(P, rule, Ea, Eb, a.adet[aT], a.adet[bT], L, N, nsub);
            prime = false;
        } else if (DIM == 2) {
            vec_retriangulate<OD>(P, rule, Ea, Eb, a.adet[aT], L, N, LP, NP, a.err, nsub);
        }
        for (int ra = 0; ra < NB; ra++) {
            for (int cb = 0; cb < NB; cb++) {
                if (a.labV[aV[ra / OD]] > 0) {
                    vec_add<OD>(a, P, aV[ra / OD], ra % OD, aV[cb / OD], cb % OD, L[NB * ra + cb]);
                    vec_add<OD>(a, P, aV[ra / OD], ra % OD, bV[cb / OD], cb % OD, -N[NB * ra + cb]);
                }
                if (prime && a.labV[bV[cb / OD]] > 0) {
                    vec_add<OD>(a, P, bV[cb / OD], cb % OD, bV[ra / OD], ra % OD, LP[NB * ra + cb]);
                    vec_add<OD>(a, P, bV[cb / OD], cb % OD, aV[ra / OD], ra % OD, -NP[NB * ra + cb]);
                }
            }
        }
    }
    const unsigned tot = __reduce_add_sync(FULL, (unsigned)nsub);
    const unsigned ncl = __reduce_add_sync(FULL, close ? 1u : 0u);
    if ((threadIdx.x & 31) == 0) {
        if (tot && a.n_subtri) atomicAdd(a.n_subtri, (unsigned long long)tot);
        if (ncl && a.n_close) atomicAdd(a.n_close, (unsigned long long)ncl);
    }
}

// Expanded rows OD v + i: nonzero count (rows of vertices with label > 0; exact zeros dropped).
// One warp per expanded row.
template <int OD>
__global__ void k_vec_finish_count(const long long *__restrict__ rowptr, long long nV, const int *__restrict__ labV,
                                   const unsigned long long *__restrict__ acc, const int *__restrict__ vprob,
                                   const ProbParams *__restrict__ probs, int *__restrict__ cnt) {
    const int lane = threadIdx.x & 31;
    const long long re = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (re >= OD * nV) return;
    const long long v = re / OD;
    const int i = (int)(re % OD);
    int c = 0;
    if (labV[v] > 0) {
        const long long rb = rowptr[v], n = rowptr[v + 1] - rb;
        const long long s0 = (long long)OD * OD * rb + (long long)i * OD * n;
        const int se = probs[vprob[v]].scale_exp;
        for (long long t = lane; t < OD * n; t += 32) c += fx_to_double(acc[2 * (s0 + t)], acc[2 * (s0 + t) + 1], se) != 0.0;
    }
    c = warp_sum(c);
    if (lane == 0) cnt[re] = c;
}

template <int OD>
__global__ void k_vec_finish_compact(const long long *__restrict__ rowptr, long long nV, const int *__restrict__ labV,
                                     const int *__restrict__ cols, const unsigned long long *__restrict__ acc,
                                     const int *__restrict__ vprob, const ProbParams *__restrict__ probs,
                                     const long long *__restrict__ fptr, int *__restrict__ fcols,
                                     double *__restrict__ fvals) {
    const int lane = threadIdx.x & 31;
    const long long re = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (re >= OD * nV) return;
    const long long v = re / OD;
    const int i = (int)(re % OD);
    if (labV[v] <= 0) return;
    const long long rb = rowptr[v], n = rowptr[v + 1] - rb;
    const long long s0 = (long long)OD * OD * rb + (long long)i * OD * n;
    const int se = probs[vprob[v]].scale_exp;
    long long out = fptr[re];
    for (long long t0 = 0; t0 < OD * n; t0 += 32) {
        const long long t = t0 + lane;
        double val = 0.0;
        if (t < OD * n) val = fx_to_double(acc[2 * (s0 + t)], acc[2 * (s0 + t) + 1], se);
        const bool nz = val != 0.0;
        const unsigned m = __ballot_sync(FULL, nz);
        if (nz) {
            const long long o = out + __popc(m & lanemask_lt());
            fcols[o] = OD * cols[rb + t / OD] + (int)(t % OD);
            fvals[o] = val;
        }
        out += __popc(m);
    }
}

// par_forcing / compute_f (Cassemble.cpp:149-164, 857-928) of a vector forcing: fd[OD v + o] +=
// psi_a f_o(x) |aT| dx, rows of vertices with label > 0; 1 / zeta under domain decomposition.
template <int DIM, int OD>
__global__ void k_forcing_vec(const double *__restrict__ EC, const double *__restrict__ adet,
                              const int *__restrict__ labT, const int *__restrict__ T32,
                              const int *__restrict__ labV, const int *__restrict__ eprob,
                              const ProbParams *__restrict__ probs, long long nE, Rule rule,
                              const long long *__restrict__ zptr, const long long *__restrict__ zidx,
                              unsigned long long *__restrict__ facc, unsigned *__restrict__ tiny) {
    constexpr int dV = DIM + 1;
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= nE || labT[e] <= 0) return;
    const ProbParams &P = probs[eprob[e]];
    const double *E = &EC[e * DIM * dV];
    double termf[dV * OD];
#pragma unroll
    for (int a = 0; a < dV * OD; a++) termf[a] = 0;
    for (int a = 0; a < dV * OD; a++)
        for (int i = 0; i < rule.nPx; i++) {
            double x[DIM], f[3];
            xtoPhys<DIM>(E, &rule.Px[DIM * i], x);
            load_vec_f64(P.load, x, f);
            termf[a] += rule.psix[dV * i + a / OD] * f[a % OD] * adet[e] * rule.dx[i];
        }
    const double w = P.zeta ? zeta_weight(zptr, zidx, e, e) : 1.0;
    for (int a = 0; a < dV * OD; a++) {
        const int v = T32[e * dV + a / OD];
        const long long r = (long long)OD * v + a % OD;
        if (labV[v] > 0) fx_atomic_add(&facc[2 * r], termf[a] * w, P.scale_exp, &tiny[r]);
    }
}

}  // namespace nlg
