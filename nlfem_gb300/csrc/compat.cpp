// par_assemble twins: the C entry nlfem_par_assemble and the C++ Cassemble signatures
// (include/Cassemble.h:62-71, 125-140 of the reference) on top of the GPU library. Output goes
// through the reference's file protocol so the unchanged Cython module can read it back:
//   "system":  ARMA_SPM_BIN_FN008, "K K nnz", nnz f64 values, nnz u64 row indices,
//              K+1 u64 column pointers, holding A^T in CSC (= A in CSR), nlfem.pyx:60-101
//   "forcing": ARMA_MAT_BIN_FN008, "K 1", K f64 values, nlfem.pyx:28-58
#include "../../include/nlfem_gpu.h"
#include "../../include/Cassemble_compat.h"

#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

static int write_spmat(const char *path, const nlfem_csr &A) {
    FILE *f = fopen(path, "wb");
    if (!f) return NLFEM_ERR_INVALID;
    fprintf(f, "ARMA_SPM_BIN_FN008\n%ld %ld %ld\n", A.K, A.K, A.nnz);
    fwrite(A.values, sizeof(double), (size_t)A.nnz, f);
    std::vector<unsigned long long> u((size_t)A.nnz > (size_t)(A.K + 1) ? (size_t)A.nnz : (size_t)(A.K + 1));
    for (long i = 0; i < A.nnz; i++) u[i] = (unsigned long long)A.indices[i];
    fwrite(u.data(), sizeof(unsigned long long), (size_t)A.nnz, f);
    for (long i = 0; i <= A.K; i++) u[i] = (unsigned long long)A.indptr[i];
    fwrite(u.data(), sizeof(unsigned long long), (size_t)(A.K + 1), f);
    fclose(f);
    return NLFEM_OK;
}

static int write_mat(const char *path, const double *v, long K) {
    FILE *f = fopen(path, "wb");
    if (!f) return NLFEM_ERR_INVALID;
    fprintf(f, "ARMA_MAT_BIN_FN008\n%ld 1\n", K);
    fwrite(v, sizeof(double), (size_t)K, f);
    fclose(f);
    return NLFEM_OK;
}

extern "C" int nlfem_par_assemble(
    const char *compute, const char *path_spAd, const char *path_fd, int K_Omega, int K,
    const long *ptrTriangles, const long *ptrLabelTriangles, const double *ptrVerts,
    const long *ptrLabelVerts, int nE, int nE_Omega, int nV, int nV_Omega, const double *Px, int nPx,
    const double *dx, const double *Py, int nPy, const double *dy, double sqdelta,
    int is_DiscontinuousGalerkin, int is_NeumannBoundary, const char *str_model_kernel,
    const char *str_model_f, const char *str_integration_method_remote,
    const char *str_integration_method_close, int is_PlacePointOnCap, int dim, int outdim,
    const long *ptrZetaIndicator_indices, const long *ptrZetaIndicator_indptr, long nZeta,
    const double *Pg, int degree, const double *dg, double maxDiameter, double fractional_s,
    int is_fullConnectedComponentSearch, int verbose) {
    (void)K_Omega; (void)nV_Omega; (void)is_NeumannBoundary; (void)maxDiameter;
    std::string comp(compute ? compute : "");
    // chk_Mesh (checks.cpp:49-85)
    long chk = 0;
    for (long k = 0; k < nE; k++) chk += ptrLabelTriangles[k] > 0;
    if (comp == "system" && chk != nE_Omega) return NLFEM_ERR_INVALID;
    if (!is_DiscontinuousGalerkin && (long)outdim * nV != K) return NLFEM_ERR_INVALID;
    if (is_DiscontinuousGalerkin && (long)outdim * (dim + 1) * nE != K) return NLFEM_ERR_INVALID;
    nlfem_problem p;
    memset(&p, 0, sizeof(p));
    p.dim = dim; p.outdim = outdim; p.is_dg = is_DiscontinuousGalerkin;
    p.nE = nE; p.nV = nV;
    p.elements = ptrTriangles; p.elementLabels = ptrLabelTriangles;
    p.vertices = ptrVerts; p.vertexLabels = ptrLabelVerts;
    p.Px = Px; p.nPx = nPx; p.dx = dx; p.Py = Py; p.nPy = nPy; p.dy = dy;
    p.Pg = Pg; p.tensorGaussDegree = degree; p.dg = dg;
    p.sqdelta = sqdelta; p.fractional_s = fractional_s;
    p.kernel = str_model_kernel; p.forcing = str_model_f;
    p.method_remote = str_integration_method_remote;
    p.method_close = str_integration_method_close;
    p.is_PlacePointOnCap = is_PlacePointOnCap;
    p.is_fullConnectedComponentSearch = is_fullConnectedComponentSearch;
    p.precision = NLFEM_PREC_FP64;
    p.verbose = verbose;
    p.zeta_indices = ptrZetaIndicator_indices;
    p.zeta_indptr = ptrZetaIndicator_indptr;
    p.nZeta = nZeta;
    if (comp == "system") {
        nlfem_csr A;
        memset(&A, 0, sizeof(A));
        int r = nlfem_stiffness_matrix(&p, &A);
        if (r) return r;
        r = write_spmat(path_spAd, A);
        nlfem_csr_free(&A);
        return r;
    }
    if (comp == "forcing") {
        std::vector<double> fd((size_t)K, 0.0);
        int r = nlfem_load_vector(&p, fd.data());
        if (r) return r;
        return write_mat(path_fd, fd.data(), K);
    }
    return NLFEM_ERR_INVALID;
}

// ---------------------------------------------------------------- C++ Cassemble signatures
static void die_on(int r, const char *where) {
    if (r == NLFEM_OK) return;
    fprintf(stderr, "ERROR in %s: %s (status %d)\n", where, nlfem_last_error(), r);
    abort();   // the reference aborts on every input error (checks.cpp:15-24)
}

void par_assemble(std::string compute, std::string path_spAd, std::string path_fd, int K_Omega, int K,
                  const long *ptrTriangles, const long *ptrLabelTriangles, const double *ptrVerts,
                  const long *ptrLabelVerts, int nE, int nE_Omega, int nV, int nV_Omega,
                  const double *Px, int nPx, const double *dx, const double *Py, int nPy,
                  const double *dy, double sqdelta, int is_DiscontinuousGalerkin,
                  int is_NeumannBoundary, std::string str_model_kernel, std::string str_model_f,
                  std::string str_integration_method_remote,
                  std::string str_integration_method_close, int is_PlacePointOnCap, int dim,
                  int outdim, const long *ptrZetaIndicator_indices,
                  const long *ptrZetaIndicator_indptr, long nZeta, const double *Pg, int degree,
                  const double *dg, double maxDiameter, double fractional_s,
                  int is_fullConnectedComponentSearch, int verbose) {
    int r = nlfem_par_assemble(compute.c_str(), path_spAd.c_str(), path_fd.c_str(), K_Omega, K,
                               ptrTriangles, ptrLabelTriangles, ptrVerts, ptrLabelVerts, nE,
                               nE_Omega, nV, nV_Omega, Px, nPx, dx, Py, nPy, dy, sqdelta,
                               is_DiscontinuousGalerkin, is_NeumannBoundary,
                               str_model_kernel.c_str(), str_model_f.c_str(),
                               str_integration_method_remote.c_str(),
                               str_integration_method_close.c_str(), is_PlacePointOnCap, dim,
                               outdim, ptrZetaIndicator_indices, ptrZetaIndicator_indptr, nZeta,
                               Pg, degree, dg, maxDiameter, fractional_s,
                               is_fullConnectedComponentSearch, verbose);
    die_on(r, "par_assemble");
}

int method_retriangulate(const double *xCenter, const double *TE, double sqdelta,
                         double *reTriangleList, int isPlacePointOnCap) {
    int r = nlfem_method_retriangulate(xCenter, TE, sqdelta, reTriangleList, isPlacePointOnCap);
    if (r < 0) die_on(-r, "method_retriangulate");
    return r;
}

// par_evaluateMass (Cassemble.cpp:166-246) through nlfem_evaluate_mass. The signature carries no
// element or vertex count: the first J elements are the ones read (K_Omega is unused, as in the
// reference), and for CG the vertex count is one past the largest vertex index they use. Like the
// reference it adds M ud to vd.
void par_evaluateMass(double *vd, const double *ud, long *Elements, const long *ElementLabels,
                      const double *Verts, const long *VertexLabels, int K_Omega, int J, int nP,
                      double *P, const double *dx, int dim, int outdim, int is_DiscontinuousGalerkin) {
    (void)K_Omega;
    if (J <= 0) return;
    const long dV = dim + 1;
    long nV = 0;
    for (long i = 0; i < (long)J * dV; i++) nV = std::max(nV, Elements[i] + 1);
    const long K = is_DiscontinuousGalerkin ? dV * J : nV;
    std::vector<double> Md((size_t)K * outdim, 0.0);
    die_on(nlfem_evaluate_mass(dim, outdim, is_DiscontinuousGalerkin, J, J, nV, Elements, ElementLabels, Verts,
                               VertexLabels, nP, P, dx, ud, Md.data()),
           "par_evaluateMass");
    for (size_t i = 0; i < Md.size(); i++) vd[i] += Md[i];
}

void toRef(const double *E, const double *phys_x, double *ref_p) {
    die_on(nlfem_toRef(E, phys_x, ref_p), "toRef");
}

void toPhys(const double *E, const double *p, int dim, double *out_x) {
    die_on(nlfem_toPhys(E, p, dim, out_x), "toPhys");
}

// The 2D overload toPhys(E, p, out) (Cassemble.h:69, mathhelpers.cpp:210-215).
void toPhys(const double *E, const double *p, double *out_x) {
    die_on(nlfem_toPhys(E, p, 2, out_x), "toPhys");
}

// method_retriangulateInfty (Cassemble.h:65-67, Cassemble.pxd:35-37): the reference triangulates the
// L-infinity ball with CGAL; this library has no L-infinity ball, so the call aborts with a message,
// as the reference aborts on an option it lacks. It is exported so that modules compiled against
// the reference's Cassemble.pxd (which declares it) link unchanged.
int method_retriangulateInfty(const double *, const double *, double, double *, int) {
    fprintf(stderr, "ERROR in method_retriangulateInfty: the L-infinity ball is not implemented in this library\n");
    abort();
}

void solve2x2(const double *A, const double *b, double *x) {
    die_on(nlfem_solve2x2(A, b, x), "solve2x2");
}
