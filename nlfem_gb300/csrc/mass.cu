// Mass-matrix product for the convergence-rate check: nlfem_evaluate_mass.
//
// par_evaluateMass (Cassemble.cpp:166-246) computes vd = M ud with the P1 mass matrix M of the
// first J elements whose label is positive. It integrates psi_a psi_b |det| by the rule (P, dx).
// Continuous Galerkin rows and columns belong to vertices with a positive label; discontinuous
// Galerkin indices are dV * element + a, with all rows kept. The reference adds every product with
// an OpenMP atomic. Here one thread per element adds its rows' sums into a 128-bit fixed-point
// accumulator, so the result does not depend on the order the atomics land in. The scale is an
// upper bound of every entry: the vertices' bounding-box volume times max |ud| times 2.
#include "../../include/nlfem_gpu.h"
#include "geometry.cuh"
#include "primitives.cuh"

#include <cuda_runtime.h>
#include <cmath>
#include <vector>

// sets the message that nlfem_last_error returns (defined beside it, not exported)
__attribute__((visibility("hidden"))) int nlfem_fail_internal(int code, const char *msg);

namespace {

using namespace nlg;

template <int DIM>
__global__ void k_mass(const long long *__restrict__ T, const long long *__restrict__ labT,
                       const double *__restrict__ V, const long long *__restrict__ labV, long long J, int nP,
                       const double *__restrict__ psi, const double *__restrict__ dx, int outdim, int dg,
                       const double *__restrict__ ud, int scale_exp, unsigned long long *__restrict__ acc,
                       unsigned *__restrict__ tiny) {
    constexpr int dV = DIM + 1;
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= J || labT[e] <= 0) return;
    long long idx[dV];
    bool keep[dV];
    double E[DIM * dV];
#pragma unroll
    for (int a = 0; a < dV; a++) {
        const long long v = T[e * dV + a];
        idx[a] = dg ? dV * e + a : v;
        keep[a] = dg || labV[v] > 0;
#pragma unroll
        for (int j = 0; j < DIM; j++) E[DIM * a + j] = V[v * DIM + j];
    }
    // absDet with the cofactor determinant (mathhelpers.cpp:112-129)
    double det;
    if (DIM == 2) {
        det = xsub(xmul(xsub(E[2], E[0]), xsub(E[5], E[1])), xmul(xsub(E[3], E[1]), xsub(E[4], E[0])));
    } else {
        double M[3][3];
        for (int i = 1; i < 4; i++)
            for (int j = 0; j < 3; j++) M[j][i - 1] = xsub(E[j + 3 * i], E[j]);
        const double c0 = xsub(xmul(M[1][1], M[2][2]), xmul(M[1][2], M[2][1]));
        const double c1 = xsub(xmul(M[1][0], M[2][2]), xmul(M[1][2], M[2][0]));
        const double c2 = xsub(xmul(M[1][0], M[2][1]), xmul(M[1][1], M[2][0]));
        det = xadd(xsub(xmul(M[0][0], c0), xmul(M[0][1], c1)), xmul(M[0][2], c2));
    }
    det = fabs(det);
    for (int a = 0; a < dV; a++) {
        if (!keep[a]) continue;
        for (int aOut = 0; aOut < outdim; aOut++) {
            double s = 0.0;
            for (int b = 0; b < dV; b++) {
                if (!keep[b]) continue;
                double m = 0.0;
                for (int j = 0; j < nP; j++) m += psi[j * dV + a] * psi[j * dV + b] * det * dx[j];
                for (int bOut = 0; bOut < outdim; bOut++) s += m * ud[outdim * idx[b] + bOut];
            }
            fx_atomic_add(&acc[2 * (outdim * idx[a] + aOut)], s, scale_exp, tiny);
        }
    }
}

__global__ void k_mass_finish(const unsigned long long *__restrict__ acc, long long n, int scale_exp,
                              double *__restrict__ vd) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) vd[i] = fx_to_double(acc[2 * i], acc[2 * i + 1], scale_exp);
}

unsigned grid_of(long long n, int b) { return (unsigned)((n + b - 1) / b); }

struct DevMem {   // device buffers of one call, freed on every exit path
    std::vector<void *> p;
    ~DevMem() {
        for (void *q : p) cudaFree(q);
    }
    template <typename X>
    X *get(size_t n) {
        void *q = nullptr;
        if (cudaMalloc(&q, n * sizeof(X) + 16) != cudaSuccess) return nullptr;
        p.push_back(q);
        return (X *)q;
    }
};

}  // namespace

extern "C" int nlfem_evaluate_mass(int dim, int outdim, int is_dg, long nE, long J, long nV,
                                   const long *elements, const long *elementLabels, const double *vertices,
                                   const long *vertexLabels, int nP, const double *P, const double *dx,
                                   const double *ud, double *vd) {
    if (dim != 2 && dim != 3) return nlfem_fail_internal(NLFEM_ERR_INVALID, "dim must be 2 or 3");
    if (outdim < 1 || nE <= 0 || nV <= 0 || J < 0 || J > nE || nP <= 0 || !elements || !elementLabels ||
        !vertices || !vertexLabels || !P || !dx || !ud || !vd)
        return nlfem_fail_internal(NLFEM_ERR_INVALID, "bad evaluate_mass argument");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return nlfem_fail_internal(NLFEM_ERR_CUDA, "no CUDA device");
    }
    const int dV = dim + 1;
    for (long long i = 0; i < (long long)nE * dV; i++)   // the kernel indexes vertices by these
        if (elements[i] < 0 || elements[i] >= nV)
            return nlfem_fail_internal(NLFEM_ERR_INVALID, "element vertex index out of range");
    const long long K = is_dg ? (long long)dV * nE : (long long)nV;
    const long long n = K * outdim;
    // psi[j * dV + a] = model_basisFunction (MeshTypes.cpp:16-24) at the rule's points
    std::vector<double> psi((size_t)nP * dV);
    for (int j = 0; j < nP; j++) {
        double s = 0.0;
        for (int c = 0; c < dim; c++) {
            psi[(size_t)j * dV + 1 + c] = P[dim * j + c];
            s += P[dim * j + c];
        }
        psi[(size_t)j * dV] = 1.0 - s;
    }
    // fixed-point scale: |vd| <= (sum of the elements' measures) max |ud| <= box volume max |ud|
    double umax = 0.0, vol = 1.0;
    for (long long i = 0; i < n; i++) umax = fmax(umax, fabs(ud[i]));
    for (int c = 0; c < dim; c++) {
        double lo = vertices[c], hi = vertices[c];
        for (long v = 1; v < nV; v++) {
            lo = fmin(lo, vertices[(size_t)v * dim + c]);
            hi = fmax(hi, vertices[(size_t)v * dim + c]);
        }
        vol *= fmax(hi - lo, 1e-300);
    }
    const double bound = 2.0 * vol * fmax(umax, 1e-300) * outdim;
    if (!std::isfinite(bound)) return nlfem_fail_internal(NLFEM_ERR_NUMERIC, "non-finite input to evaluate_mass");
    const int scale_exp = exact_ceil_log2(bound);
    DevMem m;
    long long *dT = m.get<long long>((size_t)nE * dV), *dLT = m.get<long long>(nE), *dLV = m.get<long long>(nV);
    double *dVx = m.get<double>((size_t)nV * dim), *dpsi = m.get<double>(psi.size()), *ddx = m.get<double>(nP);
    double *dud = m.get<double>(n), *dvd = m.get<double>(n);
    unsigned long long *acc = m.get<unsigned long long>(2 * n);
    unsigned *tiny = m.get<unsigned>(1);
    if (!dT || !dLT || !dLV || !dVx || !dpsi || !ddx || !dud || !dvd || !acc || !tiny)
        return nlfem_fail_internal(NLFEM_ERR_NOMEM, "device allocation failed");
    cudaMemcpy(dT, elements, sizeof(long long) * nE * dV, cudaMemcpyHostToDevice);
    cudaMemcpy(dLT, elementLabels, sizeof(long long) * nE, cudaMemcpyHostToDevice);
    cudaMemcpy(dLV, vertexLabels, sizeof(long long) * nV, cudaMemcpyHostToDevice);
    cudaMemcpy(dVx, vertices, sizeof(double) * nV * dim, cudaMemcpyHostToDevice);
    cudaMemcpy(dpsi, psi.data(), sizeof(double) * psi.size(), cudaMemcpyHostToDevice);
    cudaMemcpy(ddx, dx, sizeof(double) * nP, cudaMemcpyHostToDevice);
    cudaMemcpy(dud, ud, sizeof(double) * n, cudaMemcpyHostToDevice);
    cudaMemset(acc, 0, sizeof(unsigned long long) * 2 * n);
    cudaMemset(tiny, 0, sizeof(unsigned));
    if (J > 0) {
        if (dim == 2)
            k_mass<2><<<grid_of(J, 128), 128>>>(dT, dLT, dVx, dLV, J, nP, dpsi, ddx, outdim, is_dg, dud, scale_exp, acc, tiny);
        else
            k_mass<3><<<grid_of(J, 128), 128>>>(dT, dLT, dVx, dLV, J, nP, dpsi, ddx, outdim, is_dg, dud, scale_exp, acc, tiny);
    }
    k_mass_finish<<<grid_of(n, 256), 256>>>(acc, n, scale_exp, dvd);
    if (cudaMemcpy(vd, dvd, sizeof(double) * n, cudaMemcpyDeviceToHost) != cudaSuccess) {
        const char *s = cudaGetErrorString(cudaGetLastError());
        return nlfem_fail_internal(NLFEM_ERR_CUDA, s);
    }
    return NLFEM_OK;
}
