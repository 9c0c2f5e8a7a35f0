// Allocation-free load vector: nlfem_load_vector_noalloc.
//
// The ordinary entry points allocate device buffers on every call (grow-only session buffers,
// torch-free cudaMalloc). Some callers cannot let a library allocate at that moment: hosts that
// reserve all device memory for their own pool up front, real-time loops that forbid allocation
// after start-up, and plugins running inside another program that owns the device memory. This
// entry point serves them for the load vector: mesh and result are device pointers owned by the
// caller, and the only scratch (two 64-bit words of fixed-point accumulator per vertex plus a small
// header) lives in the file-scope array g_noalloc_scratch, 16 MiB on every GPU that loads the
// library, held until the process exits. No cudaMalloc, cudaFree or allocating library routine is
// called.
//
// Limits: at most NOALLOC_MAX_VERTICES (1,048,576) vertices, continuous P1 only; larger meshes are
// rejected with NLFEM_ERR_INVALID. All calls share the one array: each call clears the part it
// uses before it starts, and calls that overlap on the GPU (two streams, or two host threads)
// race on it, so the caller must serialize them. The first call on a device does a one-time set-up
// with that device current: it loads every kernel of this entry point (under lazy module loading a
// kernel's first launch can allocate) and looks up the array's device address with
// cudaGetSymbolAddress. That first call should come before any stream capture. A device whose
// context was torn down and made anew (cudaDeviceReset) gets the set-up again on its next call.
// The call returns after the result is in d_fd.
//
// Result: bit-identical to nlfem_load_vector. compute_f (Cassemble.cpp:149-164) per element, the
// same exact FP64 geometry, and the same 128-bit fixed-point sum whose scale follows the same rule
// (bounding box of the vertices, volume per element), evaluated here on the device.
#include "../../include/nlfem_gpu.h"
#include "geometry.cuh"
#include "primitives.cuh"

#include <cuda_runtime.h>
#include <math.h>
#include <mutex>
#include <string.h>
#include <string>

// sets the message that nlfem_last_error returns (defined beside it, not exported)
__attribute__((visibility("hidden"))) int nlfem_fail_internal(int code, const char *msg);

namespace {

using namespace nlg;

constexpr long long NOALLOC_MAX_VERTICES = 1LL << 20;
constexpr int NOALLOC_MAXQ = 32;
// header words after the accumulators: [0,3) bbox min, [3,6) bbox max (order-preserving
// encodings), 6 the fixed-point scale exponent (+4096), 7 the bad-index flag
constexpr long long HDR = 2 * NOALLOC_MAX_VERTICES;

static __device__ __align__(256) unsigned long long g_noalloc_scratch[2 * NOALLOC_MAX_VERTICES + 32];

struct NoallocRule {
    int nPx;
    double Px[NOALLOC_MAXQ * 3], dx[NOALLOC_MAXQ], psix[NOALLOC_MAXQ * 4];
};

__device__ __forceinline__ unsigned long long ord_enc(double x) {
    unsigned long long u = (unsigned long long)__double_as_longlong(x);
    return (u >> 63) ? ~u : (u | (1ULL << 63));
}
__device__ __forceinline__ double ord_dec(unsigned long long u) {
    return __longlong_as_double((long long)((u >> 63) ? (u & ~(1ULL << 63)) : ~u));
}

__global__ void k_noalloc_clear(unsigned long long *__restrict__ s, long long nV) {
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < 2 * nV) s[i] = 0ULL;
    if (i < 3) {
        s[HDR + i] = ord_enc(1e300);       // running minimum starts where the host rule starts
        s[HDR + 3 + i] = ord_enc(-1e300);
    }
    if (i == 0) { s[HDR + 6] = 0ULL; s[HDR + 7] = 0ULL; }
}

// Bounding box of the vertices (NaN coordinates are skipped, as std::min/std::max skip them there).
template <int DIM>
__global__ void k_noalloc_bbox(const double *__restrict__ V, long long nV, unsigned long long *__restrict__ s) {
    long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const unsigned lane = threadIdx.x & 31;
#pragma unroll
    for (int j = 0; j < DIM; j++) {
        unsigned long long lo = ~0ULL, hi = 0ULL;
        if (v < nV) {
            const double x = V[v * DIM + j];
            if (x == x) { lo = hi = ord_enc(x); }
        }
#pragma unroll
        for (int o = 16; o; o >>= 1) {
            lo = min(lo, __shfl_xor_sync(0xffffffffu, lo, o));
            hi = max(hi, __shfl_xor_sync(0xffffffffu, hi, o));
        }
        if (lane == 0) {
            if (lo != ~0ULL) atomicMin(&s[HDR + j], lo);
            if (hi != 0ULL) atomicMax(&s[HDR + 3 + j], hi);
        }
    }
}

// Scale exponent ceil(log2(mag)) with mag = 2 (max|x| + 2) * vol / nE, the rule of the load-vector
// path, in round-to-nearest steps without contraction; the ceiling is taken exactly from frexp.
template <int DIM>
__global__ void k_noalloc_scale(long long nE, unsigned long long *__restrict__ s) {
    double vol = 1.0, fm = 1.0;
#pragma unroll
    for (int j = 0; j < DIM; j++) {
        const double lo = ord_dec(s[HDR + j]), hi = ord_dec(s[HDR + 3 + j]);
        const double d = __dsub_rn(hi, lo);
        vol = __dmul_rn(vol, d < 1e-300 ? 1e-300 : d);
        const double a = fabs(lo), b = fabs(hi);
        const double m = a < b ? b : a;
        fm = fm < m ? m : fm;
    }
    const double el = __ddiv_rn(vol, (double)nE);
    double mag = __dmul_rn(__dmul_rn(2.0, __dadd_rn(fm, 2.0)), el);
    if (!(mag > 0) || !isfinite(mag)) mag = 1.0;
    s[HDR + 6] = (unsigned long long)(long long)(exact_ceil_log2(mag) + 4096);
}

// termf[a] of compute_f (Cassemble.cpp:149-164), summed over the elements with label > 0 into the
// rows of vertices with label > 0 (par_forcing, Cassemble.cpp:857-928).
template <int DIM>
__global__ void k_noalloc_forcing(const long *__restrict__ T, const long *__restrict__ labT,
                                  const double *__restrict__ V, const long *__restrict__ labV,
                                  long long nE, long long nV, NoallocRule rule, int load,
                                  unsigned long long *__restrict__ s) {
    constexpr int dV = DIM + 1;
    long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= nE || labT[e] <= 0) return;
    long vid[dV];
    double E[DIM * dV];
#pragma unroll
    for (int k = 0; k < dV; k++) {
        vid[k] = T[e * dV + k];
        if (vid[k] < 0 || vid[k] >= nV) {
            atomicOr(&s[HDR + 7], 1ULL);
            return;
        }
    }
#pragma unroll
    for (int k = 0; k < dV; k++)
#pragma unroll
        for (int j = 0; j < DIM; j++) E[DIM * k + j] = V[vid[k] * DIM + j];
    double det;   // absDet (mathhelpers.cpp:112-129), cofactor form
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
    const double adet = fabs(det);
    double termf[dV];
#pragma unroll
    for (int a = 0; a < dV; a++) termf[a] = 0;
    for (int i = 0; i < rule.nPx; i++) {
        double x[DIM];
        xtoPhys<DIM>(E, &rule.Px[DIM * i], x);
        const double fv = load_f64(load, x);
#pragma unroll
        for (int a = 0; a < dV; a++) termf[a] += rule.psix[dV * i + a] * fv * adet * rule.dx[i];
    }
    const int scale = (int)(long long)s[HDR + 6] - 4096;
#pragma unroll
    for (int a = 0; a < dV; a++)
        if (labV[vid[a]] > 0) fx_atomic_add(&s[2 * (long long)vid[a]], termf[a], scale, nullptr);
}

__global__ void k_noalloc_finish(const unsigned long long *__restrict__ s, long long nV, double *__restrict__ fd) {
    long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= nV) return;
    fd[v] = fx_to_double(s[2 * v], s[2 * v + 1], (int)(long long)s[HDR + 6] - 4096);
}

std::mutex g_lock;
void *g_addr[1024];                 // device address of g_noalloc_scratch, per device ordinal
unsigned long long g_ctx[1024];     // the context it belongs to (driver context ID, never reused)

unsigned grid_of(long long n, int b) { return (unsigned)((n + b - 1) / b); }

// The ID of the current context, from the driver's cuCtxGetCurrent and cuCtxGetId (looked up once
// through the runtime, so the library needs no link to the driver library).
cudaError_t context_id(int dev, unsigned long long *id) {
    typedef int (*get_current_t)(void **);
    typedef int (*get_id_t)(void *, unsigned long long *);
    static get_current_t get_current = nullptr;
    static get_id_t get_id = nullptr;
    if (!get_current || !get_id) {
        cudaDriverEntryPointQueryResult q1, q2;
        void *f1 = nullptr, *f2 = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f1, 12000, cudaEnableDefault, &q1) != cudaSuccess ||
            cudaGetDriverEntryPointByVersion("cuCtxGetId", &f2, 12000, cudaEnableDefault, &q2) != cudaSuccess ||
            q1 != cudaDriverEntryPointSuccess || q2 != cudaDriverEntryPointSuccess || !f1 || !f2)
            return cudaErrorNotSupported;
        get_current = (get_current_t)f1;
        get_id = (get_id_t)f2;
    }
    void *c = nullptr;
    // the current device again: since CUDA 12 this makes its primary context current
    if (cudaSetDevice(dev) != cudaSuccess) return cudaErrorNoDevice;
    if (get_current(&c) != 0 || !c || get_id(c, id) != 0) return cudaErrorDeviceUninitialized;
    return cudaSuccess;
}

// Forces every kernel of this entry point to be loaded in the current context.
cudaError_t load_kernels() {
    const void *fns[] = {(const void *)k_noalloc_clear,      (const void *)k_noalloc_bbox<2>,
                         (const void *)k_noalloc_bbox<3>,     (const void *)k_noalloc_scale<2>,
                         (const void *)k_noalloc_scale<3>,    (const void *)k_noalloc_forcing<2>,
                         (const void *)k_noalloc_forcing<3>,  (const void *)k_noalloc_finish};
    for (const void *f : fns) {
        cudaFuncAttributes a;
        const cudaError_t e = cudaFuncGetAttributes(&a, f);
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

}  // namespace

extern "C" int nlfem_load_vector_noalloc(int dim, long nE, long nV, const long *d_elements,
                                         const long *d_elementLabels, const double *d_vertices,
                                         const long *d_vertexLabels, const double *Px, int nPx,
                                         const double *dx, const char *forcing, double *d_fd,
                                         void *stream) {
    if (dim != 2 && dim != 3) return nlfem_fail_internal(NLFEM_ERR_INVALID, "dim must be 2 or 3");
    if (nE <= 0 || nV <= 0 || !d_elements || !d_elementLabels || !d_vertices || !d_vertexLabels || !d_fd)
        return nlfem_fail_internal(NLFEM_ERR_INVALID, "empty mesh or null device pointer");
    if (nV > NOALLOC_MAX_VERTICES)
        return nlfem_fail_internal(NLFEM_ERR_INVALID,
                                   "nlfem_load_vector_noalloc takes at most 1048576 vertices (its static "
                                   "scratch array); use nlfem_load_vector for larger meshes");
    if (!Px || !dx || nPx <= 0 || nPx > NOALLOC_MAXQ)
        return nlfem_fail_internal(NLFEM_ERR_INVALID, "outer quadrature rule missing or longer than 32 points");
    const std::string f(forcing ? forcing : "");
    int load;
    if (f == "linear") load = LOAD_LINEAR;
    else if (f == "linear3D") load = LOAD_LINEAR3D;
    else if (f == "constant") load = LOAD_CONSTANT;
    else return nlfem_fail_internal(NLFEM_ERR_UNSUPPORTED, ("unknown forcing: " + f).c_str());

    NoallocRule rule;   // psi_a at the outer points; the checks of the ordinary path's rule set-up
    memset(&rule, 0, sizeof(rule));
    rule.nPx = nPx;
    const int dV = dim + 1;
    double sx = 0;
    for (int k = 0; k < nPx; k++) {
        double p = 1.0;
        for (int j = 0; j < dim; j++) {
            rule.Px[dim * k + j] = Px[dim * k + j];
            p -= Px[dim * k + j];
            rule.psix[dV * k + j + 1] = Px[dim * k + j];
        }
        rule.psix[dV * k] = p;
        rule.dx[k] = dx[k];
    }
    for (int k = 0; k < nPx; k++) sx += rule.dx[k] * rule.psix[dV * k];
    if (fabs(sx - (dim == 2 ? 1.0 / 6.0 : 1.0 / 24.0)) >= 1e-8)
        return nlfem_fail_internal(NLFEM_ERR_INVALID, "Wrong integral of basis function w.r.t. weights dx.");

    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 1024) {
        cudaGetLastError();
        return nlfem_fail_internal(NLFEM_ERR_CUDA, "no CUDA device available (the library has no CPU path)");
    }
    unsigned long long *s;
    {
        std::lock_guard<std::mutex> g(g_lock);
        unsigned long long ctx = 0;
        if (context_id(dev, &ctx) != cudaSuccess) {
            cudaGetLastError();
            return nlfem_fail_internal(NLFEM_ERR_CUDA, "no current CUDA context");
        }
        if (!g_addr[dev] || g_ctx[dev] != ctx) {
            // Set-up, once per device (and again if the device's context was torn down and made
            // anew, e.g. by cudaDeviceReset), with that device current: the array's device
            // address, and every kernel this entry point launches loaded now, because under lazy
            // module loading a kernel's code is loaded, and device memory possibly allocated for
            // it, at its first launch. Later calls allocate nothing.
            void *p = nullptr;
            cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
            if (e == cudaSuccess && !p) e = cudaErrorInvalidSymbol;
            if (e == cudaSuccess) e = load_kernels();
            if (e != cudaSuccess) {
                cudaGetLastError();
                return nlfem_fail_internal(NLFEM_ERR_CUDA, (std::string("set-up of the no-alloc load vector: ") +
                                                            cudaGetErrorString(e)).c_str());
            }
            g_addr[dev] = p;
            g_ctx[dev] = ctx;
        }
        s = (unsigned long long *)g_addr[dev];
    }

    cudaStream_t st = (cudaStream_t)stream;
    k_noalloc_clear<<<grid_of(2 * (long long)nV, 256), 256, 0, st>>>(s, nV);
    if (dim == 2) {
        k_noalloc_bbox<2><<<grid_of(nV, 256), 256, 0, st>>>(d_vertices, nV, s);
        k_noalloc_scale<2><<<1, 1, 0, st>>>(nE, s);
        k_noalloc_forcing<2><<<grid_of(nE, 128), 128, 0, st>>>(d_elements, d_elementLabels, d_vertices,
                                                               d_vertexLabels, nE, nV, rule, load, s);
    } else {
        k_noalloc_bbox<3><<<grid_of(nV, 256), 256, 0, st>>>(d_vertices, nV, s);
        k_noalloc_scale<3><<<1, 1, 0, st>>>(nE, s);
        k_noalloc_forcing<3><<<grid_of(nE, 128), 128, 0, st>>>(d_elements, d_elementLabels, d_vertices,
                                                               d_vertexLabels, nE, nV, rule, load, s);
    }
    k_noalloc_finish<<<grid_of(nV, 256), 256, 0, st>>>(s, nV, d_fd);
    unsigned long long bad = 0;
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(&bad, s + HDR + 7, sizeof(bad), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return nlfem_fail_internal(NLFEM_ERR_CUDA, cudaGetErrorString(e));
    if (bad) return nlfem_fail_internal(NLFEM_ERR_INVALID, "an element references a vertex index outside [0, nV)");
    return NLFEM_OK;
}
