// Driver around the reference's own C++ assembly (TEST INFRASTRUCTURE ONLY).
//
// oracle/ref.mk compiles the reference's src/Cassemble.cpp, integration.cpp, model.cpp,
// MeshTypes.cpp and mathhelpers.cpp unmodified, from where they lie, against the project-written
// stand-ins in oracle/refshim/ (an Armadillo subset, two METIS calls, CGAL types), and links them
// with this file into oracle/_ref/libnlfem_ref.so. Nothing of the reference is copied: this file
// only calls its public functions (include/Cassemble.h) and supplies what the stand-ins declare.
//
// What it exports (ctypes, plain pointers):
//   ref_par_assemble   par_assemble (Cassemble.cpp:360-462) with the reference's arguments, run on
//                      a thread with a large stack (the reference keeps eind/eptr/epart/npart as
//                      stack arrays, Cassemble.cpp:394-395, 486-487) and a chosen OpenMP thread
//                      count; pass paths "mem:<name>" to keep the results in memory
//   ref_take_sparse / ref_copy_sparse / ref_take_dense / ref_copy_dense   read those results back
//   ref_evaluate_mass, ref_retriangulate, ref_toRef, ref_toPhys, ref_solve2x2   the other
//                      functions of Cassemble.h / Cassemble.pxd:32-40
#include <Cassemble.h>

#include <omp.h>
#include <pthread.h>

#include <algorithm>
#include <chrono>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "metis.h"

namespace refshim {
static std::mutex g_mu;
static std::map<std::string, Sparse> g_sparse;
static std::map<std::string, Dense> g_dense;
void keep_sparse(const std::string &name, Sparse &&s) {
    std::lock_guard<std::mutex> g(g_mu);
    g_sparse[name] = std::move(s);
}
void keep_dense(const std::string &name, Dense &&d) {
    std::lock_guard<std::mutex> g(g_mu);
    g_dense[name] = std::move(d);
}
}  // namespace refshim

// ---- METIS stand-ins (see refshim/metis.h)

int METIS_MeshToDual(idx_t *ne, idx_t *nn, idx_t *eptr, idx_t *eind, idx_t *ncommon, idx_t *numflag,
                     idx_t **r_xadj, idx_t **r_adjncy) {
    if (*ncommon != 1 || *numflag != 0) {
        std::fprintf(stderr, "refshim METIS_MeshToDual: only ncommon = 1, numflag = 0\n");
        std::abort();
    }
    const idx_t nE = *ne, nV = *nn;
    std::vector<idx_t> vcount(nV + 1, 0);
    for (idx_t e = 0; e < nE; e++)
        for (idx_t k = eptr[e]; k < eptr[e + 1]; k++) vcount[eind[k] + 1]++;
    for (idx_t v = 0; v < nV; v++) vcount[v + 1] += vcount[v];
    std::vector<idx_t> vel(vcount[nV]), fillp(vcount.begin(), vcount.end() - 1);
    for (idx_t e = 0; e < nE; e++)
        for (idx_t k = eptr[e]; k < eptr[e + 1]; k++) vel[fillp[eind[k]]++] = e;
    std::vector<std::vector<idx_t>> nb(nE);
    idx_t total = 0;
    for (idx_t e = 0; e < nE; e++) {
        std::vector<idx_t> &l = nb[e];
        for (idx_t k = eptr[e]; k < eptr[e + 1]; k++)
            for (idx_t j = vcount[eind[k]]; j < vcount[eind[k] + 1]; j++)
                if (vel[j] != e) l.push_back(vel[j]);
        std::sort(l.begin(), l.end());
        l.erase(std::unique(l.begin(), l.end()), l.end());
        total += (idx_t)l.size();
    }
    idx_t *xadj = (idx_t *)std::malloc(sizeof(idx_t) * (nE + 1));
    idx_t *adj = (idx_t *)std::malloc(sizeof(idx_t) * std::max<idx_t>(total, 1));
    if (!xadj || !adj) return METIS_ERROR;
    xadj[0] = 0;
    for (idx_t e = 0; e < nE; e++) {
        std::copy(nb[e].begin(), nb[e].end(), adj + xadj[e]);
        xadj[e + 1] = xadj[e] + (idx_t)nb[e].size();
    }
    *r_xadj = xadj;
    *r_adjncy = adj;
    return METIS_OK;
}

int METIS_PartMeshDual(idx_t *ne, idx_t *nn, idx_t *, idx_t *, idx_t *, idx_t *, idx_t *, idx_t *nparts,
                       real_t *, idx_t *, idx_t *objval, idx_t *epart, idx_t *npart) {
    const idx_t nE = *ne, p = *nparts;
    for (idx_t e = 0; e < nE; e++) epart[e] = (idx_t)((__int128)e * p / nE);
    for (idx_t v = 0; v < *nn; v++) npart[v] = 0;
    *objval = 0;
    return METIS_OK;
}

int METIS_Free(void *ptr) {
    std::free(ptr);
    return METIS_OK;
}

// ---- par_assemble on a big-stack thread

namespace {
struct Args {
    std::string compute, path_spAd, path_fd, kernel, f, remote, close;
    int K_Omega, K;
    const long *T, *labT;
    const double *V;
    const long *labV;
    int nE, nE_Omega, nV, nV_Omega;
    const double *Px, *dx, *Py, *dy;
    int nPx, nPy;
    double sqdelta;
    int is_dg, is_neumann, caps, dim, outdim;
    const long *zeta_indices, *zeta_indptr;
    long nZeta;
    const double *Pg, *dg;
    int degree;
    double maxDiameter, s;
    int full, verbose, nthreads;
    double seconds;
};

void *run(void *p) {
    Args &a = *(Args *)p;
    if (a.nthreads > 0) omp_set_num_threads(a.nthreads);
    const auto t0 = std::chrono::steady_clock::now();
    par_assemble(a.compute, a.path_spAd, a.path_fd, a.K_Omega, a.K, a.T, a.labT, a.V, a.labV, a.nE, a.nE_Omega,
                 a.nV, a.nV_Omega, a.Px, a.nPx, a.dx, a.Py, a.nPy, a.dy, a.sqdelta, a.is_dg, a.is_neumann, a.kernel,
                 a.f, a.remote, a.close, a.caps, a.dim, a.outdim, a.zeta_indices, a.zeta_indptr, a.nZeta, a.Pg,
                 a.degree, a.dg, a.maxDiameter, a.s, a.full, a.verbose);
    a.seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    return nullptr;
}
}  // namespace

extern "C" {

// Returns the wall seconds of par_assemble, or a negative value if the thread could not start.
double ref_par_assemble(const char *compute, const char *path_spAd, const char *path_fd, int K_Omega, int K,
                        const long *T, const long *labT, const double *V, const long *labV, int nE, int nE_Omega,
                        int nV, int nV_Omega, const double *Px, int nPx, const double *dx, const double *Py,
                        int nPy, const double *dy, double sqdelta, int is_dg, int is_neumann, const char *kernel,
                        const char *f, const char *remote, const char *close, int caps, int dim, int outdim,
                        const long *zeta_indices, const long *zeta_indptr, long nZeta, const double *Pg,
                        int degree, const double *dg, double maxDiameter, double s, int full, int verbose,
                        int nthreads, long stack_mb) {
    Args a{compute, path_spAd, path_fd, kernel, f, remote, close, K_Omega, K, T, labT, V, labV, nE, nE_Omega,
           nV, nV_Omega, Px, dx, Py, dy, nPx, nPy, sqdelta, is_dg, is_neumann, caps, dim, outdim,
           zeta_indices, zeta_indptr, nZeta, Pg, dg, degree, maxDiameter, s, full, verbose, nthreads, 0.0};
    pthread_attr_t attr;
    pthread_attr_init(&attr);
    pthread_attr_setstacksize(&attr, (size_t)std::max<long>(stack_mb, 16) << 20);
    pthread_t th;
    if (pthread_create(&th, &attr, run, &a) != 0) {
        pthread_attr_destroy(&attr);
        return -1.0;
    }
    pthread_join(th, nullptr);
    pthread_attr_destroy(&attr);
    return a.seconds;
}

// Sizes of a kept sparse result (-1 if absent). The stored matrix is what the reference saves:
// A^T in compressed columns, i.e. A in compressed rows (values, column indices, row pointers).
long ref_take_sparse(const char *name, unsigned long long *n_rows, unsigned long long *n_cols) {
    std::lock_guard<std::mutex> g(refshim::g_mu);
    auto it = refshim::g_sparse.find(name);
    if (it == refshim::g_sparse.end()) return -1;
    *n_rows = it->second.n_rows;
    *n_cols = it->second.n_cols;
    return (long)it->second.values.size();
}

int ref_copy_sparse(const char *name, double *values, unsigned long long *row_indices,
                    unsigned long long *col_ptrs) {
    std::lock_guard<std::mutex> g(refshim::g_mu);
    auto it = refshim::g_sparse.find(name);
    if (it == refshim::g_sparse.end()) return -1;
    const refshim::Sparse &s = it->second;
    std::copy(s.values.begin(), s.values.end(), values);
    std::copy(s.row_indices.begin(), s.row_indices.end(), row_indices);
    std::copy(s.col_ptrs.begin(), s.col_ptrs.end(), col_ptrs);
    refshim::g_sparse.erase(it);
    return 0;
}

long ref_take_dense(const char *name, unsigned long long *n_rows, unsigned long long *n_cols) {
    std::lock_guard<std::mutex> g(refshim::g_mu);
    auto it = refshim::g_dense.find(name);
    if (it == refshim::g_dense.end()) return -1;
    *n_rows = it->second.n_rows;
    *n_cols = it->second.n_cols;
    return (long)it->second.values.size();
}

int ref_copy_dense(const char *name, double *values) {
    std::lock_guard<std::mutex> g(refshim::g_mu);
    auto it = refshim::g_dense.find(name);
    if (it == refshim::g_dense.end()) return -1;
    std::copy(it->second.values.begin(), it->second.values.end(), values);
    refshim::g_dense.erase(it);
    return 0;
}

void ref_evaluate_mass(double *vd, const double *ud, long *Elements, const long *ElementLabels, const double *Verts,
                       const long *VertexLabels, int K_Omega, int J, int nP, double *P, const double *dx, int dim,
                       int outdim, int is_dg) {
    par_evaluateMass(vd, ud, Elements, ElementLabels, Verts, VertexLabels, K_Omega, J, nP, P, dx, dim, outdim, is_dg);
}

int ref_retriangulate(const double *x, const double *TE, double sqdelta, double *out, int caps) {
    return method_retriangulate(x, TE, sqdelta, out, caps);
}

void ref_toRef(const double *E, const double *x, double *p) { toRef(E, x, p); }
void ref_toPhys(const double *E, const double *p, int dim, double *x) { toPhys(E, p, dim, x); }
void ref_solve2x2(const double *A, const double *b, double *x) { solve2x2(A, b, x); }

}  // extern "C"
