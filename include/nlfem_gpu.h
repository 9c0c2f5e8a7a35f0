/* nlfem_gpu.h - C ABI of the GB300 nonlocal assembly library (libnlfem_gpu.so).
 *
 * Drop-in boundary for nlfem's assembly path. Every entry point takes plain pointers and
 * sizes (row-major, int64 indices as the reference's `long`), returns an nlfem status code
 * instead of aborting, and runs its arithmetic on the GPU (sm_103a). No CPU fallback exists:
 * without a usable CUDA device every compute entry point returns NLFEM_ERR_CUDA (after the host
 * checks of its problems, which report a refused configuration as such on any machine).
 *
 * Reference interfaces replaced (cagau/nlfem):
 *   nlfem_par_assemble        <- par_assemble         include/Cassemble.h:125-140,
 *                                                      bound by include/Cassemble.pxd:12-25
 *   nlfem_stiffness_matrix    <- par_system           include/Cassemble.h:171 (+ nlfem.pyx:128-274
 *                                                      read-back, in memory instead of a file)
 *   nlfem_load_vector         <- par_forcing          include/Cassemble.h:182 (+ nlfem.pyx:276-389)
 *   nlfem_method_retriangulate<- method_retriangulate include/Cassemble.h:62-64, Cassemble.pxd:32-34
 *   nlfem_toRef               <- toRef                include/Cassemble.h:68, Cassemble.pxd:38
 *   nlfem_toPhys              <- toPhys(E,p,dim,out)  include/Cassemble.h:70, Cassemble.pxd:39
 *   nlfem_solve2x2            <- solve2x2             include/Cassemble.h:71, Cassemble.pxd:40
 *   nlfem_stiffness_batch     <- (no counterpart: many independent par_system calls in one pass)
 *   nlfem_pair_list           <- (no counterpart: exposes the BFS interaction pairs of par_system,
 *                                 src/Cassemble.cpp:595-783, for parity checks)
 *   nlfem_pair_blocks         <- (no counterpart: the four local blocks integrate() returns,
 *                                 src/integration.cpp:67-79, for explicit pairs)
 */
#ifndef NLFEM_GPU_H
#define NLFEM_GPU_H

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define NLFEM_OK 0
#define NLFEM_ERR_INVALID 1     /* bad argument or configuration (the reference aborts) */
#define NLFEM_ERR_CUDA 2        /* no device, launch or runtime failure */
#define NLFEM_ERR_NOMEM 3       /* device or host allocation failed */
#define NLFEM_ERR_UNSUPPORTED 4 /* option outside the implemented set */
#define NLFEM_ERR_NUMERIC 5     /* where the reference aborts: a degenerate element (solve2x2), a
                                   labeled kernel outside its cases */
#define NLFEM_ERR_TIMEOUT 6     /* a bounded device wait ran out */

/* arithmetic of the quadrature */
#define NLFEM_PREC_FP64 0       /* all FP64, the reference's arithmetic */
#define NLFEM_PREC_MIXED 1      /* FP32 quadrature, FP64 cut geometry and accumulation */
#define NLFEM_PREC_FP64_ONESIDED 2 /* FP64 arithmetic in the mixed path's algorithm (one-sided pass,
                                      closed forms, fixed-point sums): 2D retriangulate only; it
                                      measures what the precision alone costs */

/* One assembly problem. Arrays are borrowed host pointers, row-major. */
typedef struct nlfem_problem {
    int dim;                     /* 2 or 3 */
    int outdim;                  /* components of the kernel's / forcing's values: 1; 2 for "constantField",
                                    "linearPrototypeMicroelasticField" (2D) and the 2D vector forcings;
                                    3 for "linearPrototypeMicroelasticField3D" and "linearField3D".
                                    K = outdim nV rows (FP64, continuous P1, no domain decomposition) */
    int is_dg;                   /* 0: continuous P1 (K = nV), 1: discontinuous (K = nE*(dim+1);
                                    FP64, one problem per call, non-singular kernels) */
    long nE, nV;
    const long *elements;        /* (nE, dim+1) vertex indices */
    const long *elementLabels;   /* (nE,) >0 domain, <0 Dirichlet layer, 0 bridge only */
    const double *vertices;      /* (nV, dim) */
    const long *vertexLabels;    /* (nV,) rows with label <= 0 are not assembled (CG) */
    const double *Px; int nPx; const double *dx;   /* outer rule on the reference element */
    const double *Py; int nPy; const double *dy;   /* inner rule */
    const double *Pg; int tensorGaussDegree; const double *dg; /* [-1,1]^4 tensor rule (singular) */
    double sqdelta;              /* squared horizon */
    double fractional_s;         /* s of the fractional kernel, -1 if unused */
    const char *kernel;          /* "constant", "parabola", "fractional", "linearPrototypeMicroelastic",
                                    "constant3D"; FP64 only, 2D: "labeled", "notch", "labeledNotch",
                                    "labeledValve", "constantTruncated"; FP64 only, outdim > 1:
                                    "constantField", "linearPrototypeMicroelasticField",
                                    "linearPrototypeMicroelasticField3D" */
    const char *forcing;         /* "linear", "linear3D", "constant", "gaussian", "jump", "tensorsin";
                                    outdim 2: "linearField", "constantRightField", "constantDownField",
                                    "constantBothField"; outdim 3: "linearField3D" */
    const char *method_remote;   /* "retriangulate", "baryCenter"; FP64 only, 2D: "retriangulate_unsymm",
                                    "subSetBall", "averageBall", "baryCenterRT", "noTruncation",
                                    "exactBall" */
    const char *method_close;    /* singular kernels: "fractional", "weakSingular" (FP64 only), or
                                    NULL (= method_remote) */
    int is_PlacePointOnCap;
    int is_fullConnectedComponentSearch;
    int precision;               /* NLFEM_PREC_FP64, NLFEM_PREC_MIXED or NLFEM_PREC_FP64_ONESIDED */
    int verbose;
    /* domain decomposition (Cassemble.cpp:649-657), nZeta > 0: element -> subdomain indicator
     * in CSR (nE + 1 row pointers, sorted column indices per row); each pair's four blocks are
     * weighted by 1 / (the number of subdomains its two elements share) */
    const long *zeta_indices;
    const long *zeta_indptr;
    long nZeta;
} nlfem_problem;

/* CSR matrix owned by the library; release with nlfem_csr_free. */
typedef struct nlfem_csr {
    long K;
    long nnz;
    long *indptr;   /* K+1 */
    long *indices;  /* nnz, ascending within a row */
    double *values; /* nnz */
} nlfem_csr;

/* The same with 32-bit row pointers and columns (matrices below 2^31 entries): the index type
 * scipy uses for such matrices, so the Python layer wraps the arrays without copying. The three
 * arrays share one pinned host block owned by the library: release it with nlfem_csr32_free
 * only (the block is kept for the next result). */
typedef struct nlfem_csr32 {
    long K;
    long nnz;
    int *indptr;    /* K+1 */
    int *indices;   /* nnz, ascending within a row */
    double *values; /* nnz */
} nlfem_csr32;

/* Run statistics of the last assembly on this thread. */
typedef struct nlfem_stats {
    long n_pairs;        /* interacting ordered element pairs (contributing integrate() calls) */
    long n_candidates;   /* integrate() calls of the BFS, interacting or not */
    long n_close;        /* pairs integrated with the singular close-pair rule */
    long nnz_structural; /* slots before exact zeros are dropped */
    long n_subtri;       /* (pair, outer point, sub-triangle) units of the remote rule, each once */
    long n_ambiguous;    /* outer points whose FP32 geometry fell back to FP64 (mixed precision) */
    double ms_total;     /* device time of the assembly (CUDA events) */
    double ms_bfs, ms_pattern, ms_quad, ms_finish;
    long n_launches;     /* kernels the library launched for the assembly */
    long n_items_in;     /* one-sided mixed passes: (pair, outer point) items whose ball holds the
                            inner element (retriangulate) or its barycenter (baryCenter) */
    long n_items_cut;    /* one-sided mixed retriangulate pass: items whose ball cuts the element */
    long slot_map;       /* one-sided passes: matrix slots found by 1 window-rank bitmaps (rows whose
                            column numbers span a narrow range), 2 per-row hash tables, 0 neither */
    long dev_bytes;      /* device memory the session's buffers hold after the assembly */
} nlfem_stats;

const char *nlfem_last_error(void);
int nlfem_device_count(void);
int nlfem_get_stats(nlfem_stats *out);

/* Stiffness matrix of one problem, host in / host out (the nlfem.stiffnessMatrix path). */
int nlfem_stiffness_matrix(const nlfem_problem *prob, nlfem_csr *out);
/* Load vector (K doubles written to fd; the nlfem.loadVector path). */
int nlfem_load_vector(const nlfem_problem *prob, double *fd);
/* Many independent problems in one pass; outs[i] receives problem i's matrix. */
int nlfem_stiffness_batch(const nlfem_problem *probs, int n, nlfem_csr *outs);
void nlfem_csr_free(nlfem_csr *m);
/* 32-bit variants (NLFEM_ERR_UNSUPPORTED when a matrix has 2^31 entries or more). */
int nlfem_stiffness_matrix32(const nlfem_problem *prob, nlfem_csr32 *out);
int nlfem_stiffness_batch32(const nlfem_problem *probs, int n, nlfem_csr32 *outs);
void nlfem_csr32_free(nlfem_csr32 *m);
/* The one-shot calls keep the device buffers of their last assembly for the next call on the
 * same device, and freed 32-bit results keep their pinned host blocks (no counterpart in the
 * reference); this frees both. */
void nlfem_cache_release(void);

/* par_evaluateMass (Cassemble.h:202-204): vd = M ud with the P1 mass matrix of the first J
 * elements whose label is positive, integrated by the rule (P, dx) of nP points. CG rows and
 * columns are the vertices with a positive label; DG (is_dg) indices are (dim + 1) * element + a.
 * Host arrays: elements (nE, dim + 1), elementLabels (nE), vertices (nV, dim), vertexLabels (nV),
 * ud and vd of K * outdim entries, K = nV (CG) or (dim + 1) * nE (DG). Deterministic. */
int nlfem_evaluate_mass(int dim, int outdim, int is_dg, long nE, long J, long nV, const long *elements,
                        const long *elementLabels, const double *vertices, const long *vertexLabels,
                        int nP, const double *P, const double *dx, const double *ud, double *vd);

/* Device-resident sessions: upload once, assemble many times (benchmarks, repeated solves). */
typedef struct nlfem_session nlfem_session;
int nlfem_session_create(const nlfem_problem *probs, int n, nlfem_session **out);
int nlfem_session_assemble(nlfem_session *s);            /* inputs already in HBM */
/* The same assembly replayed from a CUDA graph: the first call assembles and captures the
 * sequence, later calls launch the graph (falls back to a normal assembly when a capacity check
 * trips). Mixed-precision sessions only; other sessions assemble normally. */
int nlfem_session_assemble_graph(nlfem_session *s);
/* Launch-shape autotuner (no counterpart in the reference, whose OpenMP loops have no launch
 * shape): times the session's assembly with 1, 2, ... blocks per SM (up to the occupancy limit)
 * for the pair search and for the persistent one-sided quadrature pass, best of reps runs each,
 * keeps the fastest (ties within 1% go to fewer blocks: less search scratch), records the choice
 * for the device and configuration class (later sessions of the class start from it; with the
 * environment variable NLFEM_TUNE_FILE set, records persist in that file), and leaves the
 * session assembled with it. */
typedef struct nlfem_tuning {
    int bfs_blocks_per_sm, pass_blocks_per_sm;   /* chosen (pass: 0 for the colored and vector paths) */
    int bfs_candidates, pass_candidates;         /* candidates timed: 1 .. n blocks per SM */
    double bfs_ms[8], pass_ms[8];                /* best phase time (ms) of each candidate */
} nlfem_tuning;
int nlfem_session_autotune(nlfem_session *s, int reps, nlfem_tuning *out);
int nlfem_session_download(nlfem_session *s, int i, nlfem_csr *out);
int nlfem_session_download32(nlfem_session *s, int i, nlfem_csr32 *out);
/* A_Omega u = f_Omega - A_Gamma g by conjugate gradients on problem i's assembled matrix
 * (computeRates2D.py:47-70): unknowns are the vertices with label > 0, g holds the Dirichlet
 * values (read at label < 0). f, g and u have nV entries (host arrays); u returns the solution at
 * label > 0 and g at label < 0. Stops when |r| <= rtol |b| (NLFEM_ERR_NUMERIC after maxit
 * iterations); *iterations receives the count. Deterministic. */
int nlfem_session_solve(nlfem_session *s, int i, const double *f, const double *g, double rtol, int maxit,
                        double *u, int *iterations);
/* Testing hook of the pair search's visited stamps: sets every search warp's 16-bit stamp epoch
 * (the next outer element a warp takes uses epoch + 1; after 0xffff the warp clears its stamps
 * and starts again at 1). Needs one assembly of the session first (NLFEM_ERR_INVALID before).
 * The epoch must lie above every epoch any warp used since it last cleared its stamps (stale
 * stamps would otherwise read as visited): move it forward once, then let assemblies run. */
int nlfem_session_set_search_epoch(nlfem_session *s, unsigned epoch);
void nlfem_session_destroy(nlfem_session *s);

/* The interacting pairs (aT, bT) of the BFS, sorted by (aT, bT). Free *pairs with free(). */
int nlfem_pair_list(const nlfem_problem *prob, long *n_pairs, long **pairs);
/* Local blocks (termLocal, termNonloc, termLocalPrime, termNonlocPrime) of explicit pairs:
 * out (n, 4, dim+1, dim+1); does_interact (n,). close != 0 selects the close-pair rule. */
int nlfem_pair_blocks(const nlfem_problem *prob, long n, const long *pairs, int close,
                      double *out, int *does_interact);

/* Geometry primitives of the Python debug hooks (cython/nlfem.pyx:712-771), on the GPU. */
int nlfem_method_retriangulate(const double *x_center, const double *TE, double sqdelta,
                               double *reTriangleList, int is_placePointOnCap);
int nlfem_retriangulate_batch(long n, const double *x_center, const double *TE, double sqdelta,
                              int is_placePointOnCap, int *counts, double *reTriangleList);
/* Test hook (no counterpart in the reference): the certified FP32 retriangulation of the mixed
 * path on the same cases; ambiguous[i] != 0 marks cases it hands to the FP64 routine. points
 * (n, 9, 2) relative to the center. */
int nlfem_retriangulate_certified_batch(long n, const double *x_center, const double *TE, double sqdelta,
                                        int caps, int *counts, int *ambiguous, double *points);
int nlfem_toRef(const double *E, const double *phys_x, double *ref_p);
int nlfem_toPhys(const double *E, const double *p, int dim, double *out_x);
int nlfem_solve2x2(const double *A, const double *b, double *x);

/* C twin of par_assemble (include/Cassemble.h:125-140) with C strings. Writes the arma binary
 * files the unchanged nlfem.pyx reads back (ARMA_SPM_BIN_FN008 for "system" holding A^T in CSC,
 * ARMA_MAT_BIN_FN008 for "forcing"). Returns a status instead of aborting. */
int nlfem_par_assemble(const char *compute, const char *path_spAd, const char *path_fd,
                       int K_Omega, int K, const long *ptrTriangles, const long *ptrLabelTriangles,
                       const double *ptrVerts, const long *ptrLabelVerts, int nE, int nE_Omega,
                       int nV, int nV_Omega, const double *Px, int nPx, const double *dx,
                       const double *Py, int nPy, const double *dy, double sqdelta,
                       int is_DiscontinuousGalerkin, int is_NeumannBoundary,
                       const char *str_model_kernel, const char *str_model_f,
                       const char *str_integration_method_remote,
                       const char *str_integration_method_close, int is_PlacePointOnCap,
                       int dim, int outdim, const long *ptrZetaIndicator_indices,
                       const long *ptrZetaIndicator_indptr, long nZeta, const double *Pg,
                       int degree, const double *dg, double maxDiameter, double fractional_s,
                       int is_fullConnectedComponentSearch, int verbose);

/* Benchmark helper (no counterpart in the reference): measured FP32 and FP64 FMA throughput of
 * the current device in TFLOP/s, the roofline denominators of the quadrature kernels. */
int nlfem_measure_peaks(double *fp32_tflops, double *fp64_tflops);

/* Allocation-free load vector (no counterpart in the reference). The same result as
 * nlfem_load_vector (continuous P1, bit-identical) for callers that must not let a library allocate
 * device memory: the mesh arrays and d_fd (nV doubles) are caller-owned DEVICE pointers, Px/dx
 * and forcing are host data, and the only scratch is a static 16 MiB device array inside the
 * library, so no cudaMalloc or cudaFree happens. At most 1,048,576 vertices (NLFEM_ERR_INVALID
 * above). The first call on each device does a one-time set-up (it looks up the array's address
 * with that device current) and should come before any stream capture. Calls share the array:
 * overlapping calls (two streams or threads) race and must be serialized by the caller. Work is
 * queued on `stream` (a cudaStream_t, NULL for the default stream); returns once d_fd holds the
 * result. */
int nlfem_load_vector_noalloc(int dim, long nE, long nV, const long *d_elements,
                              const long *d_elementLabels, const double *d_vertices,
                              const long *d_vertexLabels, const double *Px, int nPx,
                              const double *dx, const char *forcing, double *d_fd, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* NLFEM_GPU_H */
