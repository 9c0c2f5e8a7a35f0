/* Cassemble_compat.h - the reference's C++ Cassemble entry points, exported by libnlfem_gpu.so
 * with their original signatures so that code compiled against the reference's
 * include/Cassemble.h (and include/Cassemble.pxd) links unchanged.
 *
 *   par_assemble          <- include/Cassemble.h:125-140 (bound at include/Cassemble.pxd:12-25)
 *   par_evaluateMass      <- include/Cassemble.h:202-204 (include/Cassemble.pxd:27-29)
 *   method_retriangulate  <- include/Cassemble.h:62-64   (include/Cassemble.pxd:32-34)
 *   toRef                 <- include/Cassemble.h:68      (include/Cassemble.pxd:38)
 *   toPhys                <- include/Cassemble.h:69-70   (include/Cassemble.pxd:39)
 *   solve2x2              <- include/Cassemble.h:71      (include/Cassemble.pxd:40)
 *   method_retriangulateInfty <- include/Cassemble.h:65-67 (include/Cassemble.pxd:35-37): exported
 *                            so that the reference's module links; it aborts (no L-infinity ball)
 *
 * Like the reference they abort() on invalid input; the C ABI in nlfem_gpu.h returns status
 * codes instead. The computation runs on the GPU. include/Cassemble.h carries the reference's
 * header name and includes this file, so the reference's cython/nlfem.pyx compiles against this
 * library unchanged (nlfem_gb300/dropin.py).
 */
#ifndef NLFEM_CASSEMBLE_COMPAT_H
#define NLFEM_CASSEMBLE_COMPAT_H
#include <string>

void par_assemble(std::string compute, std::string path_spAd, std::string path_fd, int K_Omega, int K,
                  const long *ptrTriangles, const long *ptrLabelTriangles, const double *ptrVerts,
                  const long *ptrLabelVerts, int nE, int nE_Omega, int nV, int nV_Omega,
                  const double *Px, int nPx, const double *dx, const double *Py, int nPy,
                  const double *dy, double sqdelta, int is_DiscontinuousGalerkin,
                  int is_NeumannBoundary, std::string str_model_kernel, std::string str_model_f,
                  std::string str_integration_method_remote,
                  std::string str_integration_method_close, int is_PlacePointOnCap, int dim,
                  int outdim, const long *ptrZetaIndicator_indices,
                  const long *ptrZetaIndicator_indptr, long nZeta = 0, const double *Pg = nullptr,
                  int degree = 0, const double *dg = nullptr, double maxDiameter = 0.0,
                  double fractional_s = -1.0, int is_fullConnectedComponentSearch = 0,
                  int verbose = 0);

void par_evaluateMass(double *vd, const double *ud, long *Elements, const long *ElementLabels,
                      const double *Verts, const long *VertexLabels, int K_Omega, int J, int nP,
                      double *P, const double *dx, int dim, int outdim, int is_DiscontinuousGalerkin);

int method_retriangulate(const double *xCenter, const double *TE, double sqdelta,
                         double *reTriangleList, int isPlacePointOnCap);
void toRef(const double *E, const double *phys_x, double *ref_p);
void toPhys(const double *E, const double *p, int dim, double *out_x);
void toPhys(const double *E, const double *p, double *out_x);
int method_retriangulateInfty(const double *xCenter, const double *TE, double sqdelta,
                              double *reTriangleList, int isPlacePointOnCap);
void solve2x2(const double *A, const double *b, double *x);

#endif
