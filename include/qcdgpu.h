/* qcdgpu.h -- C ABI of the GB300 Wilson-twisted-mass library.
 *
 * Part 1 re-declares the data model of qcd_lib (include/qcd.h) with the same
 * sizes, field order and meaning, so host code written against qcd_lib can
 * hand its qcd_geometry / qcd_vector / qcd_gaugeField structs to this library
 * unchanged. Part 2 exports, under their qcd_lib names and signatures, the
 * entry points of the operator-apply and solve path; each cites the reference
 * declaration it replaces. Part 3 is this library's own extension API
 * (device residency, precision, multi-RHS, serving) and carries the
 * qcdgpu_ prefix.
 *
 * Semantics shared by every Part-2 entry point:
 *  - the whole lattice lives on one GPU; P must be {1,1,1,1} and numprocs 1;
 *  - arguments and results are the caller's host arrays (v->D, u->D): an
 *    entry point uploads what it reads and, before it returns, writes its
 *    results back to host memory -- unless the object was made device
 *    resident with qcdgpu_vector_make_resident / qcdgpu_gauge_upload, in
 *    which case the device copy is authoritative (Part 3);
 *  - errors return 1 (or NaN for scalar results) with a message on stderr,
 *    as the reference does; CUDA failures are reported the same way; no
 *    entry point aborts the process;
 *  - Dv == v (in-place operator apply) is rejected with return value 1: the
 *    reference leaves it undefined (qcd_wilson.c writes Dv while it still
 *    reads neighbours of v).
 *  - not re-entrant per geometry; call from one host thread at a time.
 */
#ifndef QCDGPU_H
#define QCDGPU_H 1

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ============================ Part 1: data model ======================== */

/* scalar types, include/qcd.h:18-28 */
typedef float qcd_real_4;
typedef double qcd_real_8;
typedef char qcd_int_1;
typedef short qcd_int_2;
typedef int qcd_int_4;
typedef long qcd_int_8;
typedef unsigned char qcd_uint_1;
typedef unsigned short qcd_uint_2;
typedef unsigned int qcd_uint_4;
typedef unsigned long qcd_uint_8;

/* qcd_geometry embeds MPI handle arrays. The library never calls MPI; it only
 * needs their size. Handles are int-sized (the MPICH convention). A build
 * that includes a real <mpi.h> first must use an MPI with int handles. */
#ifndef MPI_VERSION
typedef int MPI_Request;
typedef int MPI_Datatype;
#endif

/* include/qcd.h:31-41 */
typedef struct {
  qcd_real_8 re;
  qcd_real_8 im;
} qcd_complex_16;

typedef struct {
  qcd_real_4 re;
  qcd_real_4 im;
} qcd_complex_8;

/* include/qcd.h:44-87 */
typedef struct {
  qcd_uint_8 V;                /* 4d volume */
  qcd_uint_8 V3;               /* spatial volume */
  qcd_uint_2 L[4];             /* lattice extents t,x,y,z */
  qcd_uint_8 lV;               /* local volume (== V here) */
  qcd_uint_8 lV3;
  qcd_uint_2 lL[4];
  qcd_uint_2 Pos[4];
  qcd_real_8 theta[4];         /* psi(x + L_mu) = exp(i theta_mu) psi(x) */
  qcd_uint_4 myid;
  qcd_uint_4 nproc;
  qcd_uint_4 Pplus[4];
  qcd_uint_4 Pminus[4];
  qcd_uint_8 (*plus)[4];       /* neighbour tables, periodic in the lattice */
  qcd_uint_8 (*minus)[4];
  qcd_uint_8 (*plus3d)[4];
  qcd_uint_8 (*minus3d)[4];
  qcd_uint_8 (*eo)[2];
  qcd_uint_8 startBminus[4];
  qcd_uint_8 startBplus[4];
  qcd_uint_8 startBminus3d[4];
  qcd_uint_8 startBplus3d[4];
  qcd_uint_8 boundarySize;
  qcd_uint_8 boundarySize3d;
  qcd_uint_8 *edge;
  qcd_uint_8 edgePoints;
  qcd_uint_8 *edge0;
  qcd_uint_8 edge0Points;
  MPI_Request requests[32];
  int numOfRequests;
  MPI_Datatype stypeV[4];
  MPI_Datatype rtypeV[4];
  MPI_Datatype stypeU[4];
  MPI_Datatype rtypeU[4];
  MPI_Datatype stypeT[4];
  MPI_Datatype rtypeT[4];
  MPI_Datatype stypeP[4];
  MPI_Datatype rtypeP[4];
  qcd_uint_2 initialized;
} qcd_geometry;

/* include/qcd.h:90-97: spinor D[site][spin][colour] */
typedef struct {
  qcd_complex_16 (*D)[4][3];
  qcd_complex_16 (*Bplus[4])[4][3];
  qcd_complex_16 (*Bminus[4])[4][3];
  qcd_geometry *geo;
  qcd_uint_2 initialized;
} qcd_vector;

/* include/qcd.h:119-126: links D[site][mu][row][col] */
typedef struct {
  qcd_complex_16 (*D)[4][3][3];
  qcd_complex_16 (*Bplus[4])[4][3][3];
  qcd_complex_16 (*Bminus[4])[4][3][3];
  qcd_geometry *geo;
  qcd_uint_2 initialized;
} qcd_gaugeField;

/* ===================== Part 2: qcd_lib entry points ===================== */

/* include/qcd.h:187-195 (lib/src/qcd_init.c:25,:394,:418,:614) */
int qcd_initGeometry(qcd_geometry *geo, const qcd_uint_2 L[], const qcd_uint_2 P[],
                     const qcd_real_8 theta[], const int myid, const int numprocs);
void qcd_destroyGeometry(const qcd_geometry *geo);
int qcd_initVector(qcd_vector *vec, qcd_geometry *geo);
void qcd_destroyVector(qcd_vector *vec);
int qcd_initGaugeField(qcd_gaugeField *u, qcd_geometry *geo);
void qcd_destroyGaugeField(qcd_gaugeField *u);

/* include/qcd_wilson.h:634-637 (lib/src/qcd_wilson.c:114,:351,:570,:795).
 * D = (m+4) + i tm gamma_5 - 1/2 sum_mu [(1-gamma_mu) U_mu(x) e^{i th/L} v(x+mu)
 *                                    + (1+gamma_mu) U_mu(x-mu)^+ e^{-i th/L} v(x-mu)]
 * in the chiral basis of qcd_gamma.c; Q = i gamma_5 D. The three D entry
 * points are the same operator (the reference's three implementations agree
 * to rounding). */
int qcd_applyWilsonTMOp(qcd_vector *Dv, qcd_vector *v, qcd_gaugeField *u, qcd_real_8 m, qcd_real_8 tm);
int qcd_applyWilsonTMOpNoScripts(qcd_vector *Dv, qcd_vector *v, qcd_gaugeField *u, qcd_real_8 m, qcd_real_8 tm);
int qcd_applyWilsonTMOpNoOptim(qcd_vector *Dv, qcd_vector *v, qcd_gaugeField *u, qcd_real_8 m, qcd_real_8 tm);
int qcd_applyQTMOp(qcd_vector *Dv, qcd_vector *v, qcd_gaugeField *u, qcd_real_8 m, qcd_real_8 tm);

/* include/qcd_blas.h:245-267 (lib/src/qcd_blas.c:137-492); all on the GPU */
void qcd_zeroVector(qcd_vector *vec);
void qcd_setVector(qcd_vector *vec, qcd_complex_16 c);
void qcd_copyVector(qcd_vector *dest, qcd_vector *src);
void qcd_mulVectorC(qcd_vector *vec, qcd_complex_16 c);
void qcd_scaleVector(qcd_vector *vec, qcd_real_8 r);
void qcd_subVector(qcd_vector *difference, qcd_vector *minuend, qcd_vector *subtrahend);
void qcd_addVector(qcd_vector *sum, qcd_vector *summand1, qcd_vector *summand2);
void qcd_axpyVector(qcd_vector *axpy, qcd_complex_16 a, qcd_vector *x, qcd_vector *y);
qcd_complex_16 qcd_mulAdjointVectorVector(qcd_vector *factor1, qcd_vector *factor2);
qcd_real_8 qcd_normVector(qcd_vector *vec);
/* include/qcd_gamma.h (lib/src/qcd_gamma.c:521) */
void qcd_gamma5Vector(qcd_vector *v);

/* include/qcd_wilson.h:628-633 (lib/src/qcd_wilson.c:18-103): host helpers
 * on one site's spin-colour vector [4][3]. (1 +- gamma_mu) vec for mu = 0..5
 * (gamma_4 = -gamma_0, gamma_5 in slot 5, as the reference's tables; other mu
 * leave result untouched); U vec and U^+ vec for a 3 x 3 colour matrix on
 * every spin; (mp4 + i tm gamma_5) vec; vec * phi in place. */
void qcd_onePlusGamma(qcd_complex_16 result[][3], qcd_complex_16 vec[][3], qcd_uint_2 mu);
void qcd_oneMinusGamma(qcd_complex_16 result[][3], qcd_complex_16 vec[][3], qcd_uint_2 mu);
void qcd_applyU(qcd_complex_16 result[][3], qcd_complex_16 u[][3], qcd_complex_16 vec[][3]);
void qcd_applyUDagger(qcd_complex_16 result[][3], qcd_complex_16 u[][3], qcd_complex_16 vec[][3]);
void qcd_massTerms(qcd_complex_16 result[][3], qcd_complex_16 vec[][3], qcd_real_8 mp4, qcd_real_8 tm);
void qcd_phaseMul(qcd_complex_16 vec[][3], qcd_complex_16 phi);

/* include/qcd_stochastic.h:5 (lib/src/qcd_stochastic.c:8-58): vec <- Z4
 * noise {1, i, -1, -i}, independent per site and spin-colour component, on
 * time-slice t_slice (every site when t_slice < 0; zero when t_slice is past
 * the lattice), generated on the GPU. The reference draws from GSL's ranlux;
 * this library draws every call a new vector from its own counter-based
 * stream, restarted by qcdgpu_set_noise_seed. Errors: qcdgpu_last_error. */
void qcd_z2Vector(qcd_vector *vec, int t_slice);
int qcdgpu_set_noise_seed(uint64_t seed);

/* Source construction, computed on the GPU.
 * include/qcd_smearing.h:41 (lib/src/qcd_smearing.c:209): one 3D APE step,
 * apeu_mu = Proj_SU3(u_mu + alpha * spatial staples) for mu = 1..3, temporal
 * links copied; apeu must be a different field of the same lattice.
 * include/qcd_smearing.h:39 (lib/src/qcd_smearing.c:25): one Gaussian step
 * v <- (v + alpha H v) / (1 + 6 alpha) on time-slice t.
 * include/qcd_observables.h:12 (lib/src/qcd_observables.c:15): mean
 * plaquette, 1 on the unit field (NaN on error). */
int qcd_apeSmear3d(qcd_gaugeField *apeu, qcd_gaugeField *u, qcd_real_8 alpha);
int qcd_gaussIteration3d(qcd_vector *v, qcd_gaugeField *u, qcd_real_8 alpha, qcd_uint_4 t);
qcd_real_8 qcd_calculatePlaquette(qcd_gaugeField *u);

/* include/qcd.h:16 and include/qcd_io.h:12-17: the string length the
 * drivers use and the file type codes. */
#ifndef qcd_MAX_STRING_LENGTH
#define qcd_MAX_STRING_LENGTH 256
#endif
#ifndef qcd_GF_LIME
#define qcd_GF_LIME 0
#define qcd_PROP_CMI 0
#define qcd_PROP_HMC 1
#define qcd_PROP_HMCV 2
#define qcd_PROP_LIME 3
#define qcd_SOURCE_LIME 4
#endif

/* Parameter files, include/qcd_io.h:21-22 (lib/src/qcd_io.c:83-129).
 * qcd_getParams returns the file in a malloc'd buffer (free it) with
 * *len = size + 1 and a terminating zero; NULL if it cannot be read.
 * qcd_getParam returns the text following the first occurrence of token,
 * cut at the next '<' (written into params); an empty string if the token
 * is absent (the reference returns the buffer's last bytes). */
char *qcd_getParams(char *fname, int *len);
char *qcd_getParam(char token[], char *params, int len);

/* LIME files, include/qcd_io.h:26-43 (lib/src/qcd_io.c:204-540,984-1150,
 * 1766-1950). ILDG gauge configurations (precision 64 or 32, big-endian,
 * file order t,z,y,x and link directions x,y,z,t) and ETMC spinor files
 * ("etmc-propagator-format" / "etmc-source-format" + "scidac-binary-data").
 * Writers produce FP64 files with qcd_lib's records. Differences: all of a
 * 32-bit gauge file is byte-swapped (qcd_io.c:377 swaps one time-slice's
 * worth); getGaugeField knows type qcd_GF_LIME (0) only. Return 0 or 1. */
int qcd_getGaugeLime(char *fname, qcd_gaugeField *u);
int qcd_getGaugeField(char *fname, int type, qcd_gaugeField *u);
int qcd_writeGaugeLime(char *fname, qcd_gaugeField *u, char *message);
int qcd_getVectorLime(char *fname, qcd_vector *v);
/* include/qcd_io.h:35-39 (lib/src/qcd_io.c:907-1340, dispatcher :1386): the
 * legacy propagator vector files, big-endian [x][y][z][t][spin][colour]
 * [re, im]: CMI float32 without header; HMC an ASCII line "beta kappa mu L
 * T" then float64 data of all 12 source columns (column nu * 3 + c2 read);
 * HMCV the same line and one column. The header line is read with the
 * reference's fscanf format, whose trailing newline also skips whitespace
 * bytes at the start of the data (the data offset follows it). Files
 * shorter than the vector are an error (the reference reads past their
 * end). qcd_getVector dispatches on type: qcd_PROP_CMI 0, qcd_PROP_HMC 1,
 * qcd_PROP_HMCV 2, qcd_PROP_LIME 3. */
int qcd_getVectorCMI(char *fname, qcd_uint_2 nu, qcd_uint_2 c2, qcd_vector *v);
int qcd_getVectorHMC(char *fname, qcd_uint_2 nu, qcd_uint_2 c2, qcd_vector *v);
int qcd_getVectorHMCV(char *fname, qcd_uint_2 nu, qcd_uint_2 c2, qcd_vector *v);
int qcd_getVector(char *fname, int type, qcd_uint_2 nu, qcd_uint_2 c2, qcd_vector *v);
int qcd_writeVectorLime(char *fname, int type, qcd_vector *v);
/* include/qcd_io.h:42,44 (lib/src/qcd_io.c:1685, :1951): a CMI file
 * (float32, rounded to nearest) and the writer dispatcher: qcd_PROP_CMI 0,
 * qcd_PROP_LIME 3, qcd_SOURCE_LIME 4 (the reference's HMC writer is
 * commented out). */
int qcd_writeVectorCMI(char *fname, qcd_uint_2 nu, qcd_uint_2 c2, qcd_vector *v);
int qcd_writeVector(char *fname, int type, qcd_uint_2 nu, qcd_uint_2 c2, qcd_vector *v);

/* include/qcd_communication.h:12,21 (lib/src/qcd_communication.c:20,:343).
 * One GPU holds the whole lattice: no halo exists, both are no-ops that keep
 * the reference's "communication already in flight" check. */
int qcd_communicateVectorPMGaugeP(qcd_vector *v, qcd_gaugeField *u);
void qcd_waitall(qcd_geometry *geo);

/* invert.c:20. n-step GCR with modified Gram-Schmidt on Q = i gamma_5 D,
 * m = 1/(2 kappa) - 4. The solution update includes the first basis term
 * (the algorithm of gcr.m); the shipped invert.c omits it (:52-53), which
 * qcdgpu_set_gcr_compat(1) restores. Returns 0, or EXIT_FAILURE when the
 * Krylov space degenerates (NaN norm). */
qcd_int_4 gcr(qcd_vector *sol, qcd_vector *src, qcd_gaugeField *u, qcd_real_8 kappa,
              qcd_real_8 muTM, qcd_uint_4 n, qcd_geometry *geo);

/* No reference counterpart (qcd_lib ships only GCR): BiCGstab (van der Vorst
 * 1992) on D x = b in FP64, x0 = 0, shadow residual a fixed seeded Z4 vector,
 * run until the true relative residual |b - Dx|/|b| <= tol or maxiter.
 * Same argument order as gcr(). Returns iterations (>= 0), or -1 on
 * breakdown / non-convergence / error. */
qcd_int_4 bicgstab(qcd_vector *sol, qcd_vector *src, qcd_gaugeField *u, qcd_real_8 kappa,
                   qcd_real_8 muTM, qcd_real_8 tol, qcd_uint_4 maxiter, qcd_geometry *geo);

/* No reference counterpart: CG on D^+ D x = D^+ b (FP64), stopping on the
 * true relative residual |b - Dx|/|b| <= tol. Returns iterations or -1. */
qcd_int_4 cgnr(qcd_vector *sol, qcd_vector *src, qcd_gaugeField *u, qcd_real_8 kappa,
               qcd_real_8 muTM, qcd_real_8 tol, qcd_uint_4 maxiter, qcd_geometry *geo);

/* ====================== Part 3: extension API ========================== */

/* Storage precision of a device field. */
enum {
  QCDGPU_F64 = 0,  /* 8-byte reals */
  QCDGPU_F32 = 1,  /* 4-byte reals */
  QCDGPU_F16 = 2   /* 2-byte reals; spinors carry one float norm per site */
};
/* Operator selector. */
enum {
  QCDGPU_OP_D = 0,       /* D */
  QCDGPU_OP_Q = 1,       /* i gamma_5 D */
  QCDGPU_OP_DDAG = 2,    /* D^+ */
  QCDGPU_OP_DDAGD = 3    /* D^+ D */
};
/* FP64 operator arithmetic. */
enum {
  QCDGPU_ARITH_F64 = 0,  /* native double precision */
  QCDGPU_ARITH_DF64 = 1  /* float-float (two FP32 words per real) */
};

typedef struct qcdgpu_field_s *qcdgpu_field; /* device spinor field */
typedef struct qcdgpu_gauge_s *qcdgpu_gauge; /* device gauge field */

/* last error message of this thread ("" if none) */
const char *qcdgpu_last_error(void);
/* select the CUDA stream (cudaStream_t) later calls launch on; NULL = default */
int qcdgpu_set_stream(void *stream);
/* synchronise the current stream */
int qcdgpu_sync(void);
/* restore invert.c's shipped GCR update (1) or the algorithm's (0, default) */
void qcdgpu_set_gcr_compat(int shipped);
/* arithmetic of the FP64 operator used by the qcd.h entry points, the FP64
 * solvers and qcdgpu_dslash with arith < 0. Default QCDGPU_ARITH_DF64:
 * float-float on the FP32 pipes, 3.6x the native rate on GB300 at the same
 * per-site parity (<= 1e-13); |x| below 2^-1022 counts as zero there.
 * QCDGPU_ARITH_F64 selects native IEEE double. */
int qcdgpu_set_f64_arith(int arith);
/* slabs of the pipelined host-buffer operator apply (0: automatic, the largest
 * of 24, 16, 12, 8, 6, 4, 3 dividing L_z; otherwise a divisor of L_z, >= 3);
 * a tuning knob with no reference counterpart */
int qcdgpu_set_pipeline_slabs(int S);
/* number of kernels this library launched since the process started */
uint64_t qcdgpu_kernel_launches(void);

/* Residency of the Part-2 host structs. make_resident uploads v->D once and
 * from then on the device copy is authoritative: entry points neither
 * upload nor download it. to_host / to_device copy explicitly. release
 * returns the object to per-call transfers (after copying back to host). */
int qcdgpu_vector_make_resident(qcd_vector *v);
int qcdgpu_vector_to_host(qcd_vector *v);
int qcdgpu_vector_to_device(qcd_vector *v);
int qcdgpu_vector_release(qcd_vector *v);
/* upload u->D and keep it resident (call again after changing u->D) */
int qcdgpu_gauge_upload(qcd_gaugeField *u);
int qcdgpu_gauge_release(qcd_gaugeField *u);

/* Device fields. L = {Lt, Lx, Ly, Lz}. Gauge fields store 12 reals per link
 * (third row rebuilt as the conjugate cross product of the first two) when
 * every link is in SU(3) to 1e-12, else all 18. */
int qcdgpu_gauge_create(qcdgpu_gauge *g, const int L[4], const double theta[4], int prec);
int qcdgpu_gauge_destroy(qcdgpu_gauge g);
/* host array in the qcd_gaugeField layout, float64[V][4][3][3][2] */
int qcdgpu_gauge_load(qcdgpu_gauge g, const double *host);
/* make a lower-precision copy of an existing gauge field */
int qcdgpu_gauge_convert(qcdgpu_gauge dst, qcdgpu_gauge src);
/* synthetic links exp(i eps H), H Gaussian traceless Hermitian, seeded */
int qcdgpu_gauge_synthetic(qcdgpu_gauge g, uint64_t seed, double eps);
/* copy out to the qcd_gaugeField layout */
int qcdgpu_gauge_store(qcdgpu_gauge g, double *host);
int qcdgpu_gauge_recon(qcdgpu_gauge g); /* 12 or 18 */
double qcdgpu_plaquette(qcdgpu_gauge g);

int qcdgpu_field_create(qcdgpu_field *f, const int L[4], int prec);
int qcdgpu_field_destroy(qcdgpu_field f);
/* host array in the qcd_vector layout, float64[V][4][3][2] */
int qcdgpu_field_load(qcdgpu_field f, const double *host);
int qcdgpu_field_store(qcdgpu_field f, double *host);
/* device-to-device copy with precision conversion */
int qcdgpu_field_copy(qcdgpu_field dst, qcdgpu_field src);
int qcdgpu_field_gaussian(qcdgpu_field f, uint64_t seed);
/* noise source (no reference counterpart beyond qcd_z2Vector): kind 4 = Z4
 * {1, i, -1, -i}, kind 2 = Z2 {1, -1} per spin-colour component, on
 * time-slice t_slice (all sites when negative), from the seeded stream */
int qcdgpu_field_noise(qcdgpu_field f, uint64_t seed, int t_slice, int kind);
int qcdgpu_field_point(qcdgpu_field f, const int x[4], int spin, int colour);
/* bytes of device memory the field occupies */
size_t qcdgpu_field_bytes(qcdgpu_field f);
size_t qcdgpu_gauge_bytes(qcdgpu_gauge g);
/* raw device pointer of the field's storage (for timing harnesses) */
void *qcdgpu_field_data(qcdgpu_field f);

/* out = op(in), m = 1/(2 kappa) - 4; out and in must differ; out, in and g
 * must have the same precision (FP64 fields use the FP64 arithmetic set by
 * qcdgpu_set_f64_arith unless arith >= 0 is given). */
int qcdgpu_dslash(qcdgpu_field out, qcdgpu_field in, qcdgpu_gauge g, double kappa, double mu,
                  int op, int arith);

/* BLAS-1 on device fields of equal shape (FP64 fields; reductions return
 * through host pointers after synchronising). */
int qcdgpu_axpy(qcdgpu_field out, double are, double aim, qcdgpu_field x, qcdgpu_field y);
int qcdgpu_norm2(qcdgpu_field x, double *result);
int qcdgpu_dot(qcdgpu_field a, qcdgpu_field b, double result[2]);

/* Solver parameters for qcdgpu_solve. */
typedef struct {
  int solver;        /* QCDGPU_SOLVER_* */
  int op;            /* QCDGPU_OP_D or QCDGPU_OP_Q (system matrix) */
  int inner_prec;    /* QCDGPU_F64 / F32 / F16: storage of the inner iteration */
  double tol;        /* target true relative residual |b - A x|/|b| */
  int maxiter;       /* cap on operator applications of the inner solver */
  int restart;       /* GCR basis size */
  double delta;      /* reliable-update threshold (mixed precision), e.g. 0.1 */
  /* outputs */
  int iters;         /* inner iterations performed */
  int reliable_updates;
  double true_residual;
  int status;        /* 0 converged, 1 not converged, 2 breakdown, 3 error */
} qcdgpu_solve_params;
enum {
  QCDGPU_SOLVER_GCR = 0,
  QCDGPU_SOLVER_BICGSTAB = 1,
  QCDGPU_SOLVER_CGNR = 2,
  /* CGNR on the even/odd (Schur) preconditioned system; every lattice
   * extent must be even (the periodic checkerboard). Same convergence test
   * on the full true residual. */
  QCDGPU_SOLVER_CGNR_EO = 3,
  /* BiCGstab(l) (Sleijpen-Fokkema) on the even/odd Schur complement (every
   * extent even), l =
   * restart when 1..16 (else 8); inner iterations in inner_prec with FP64
   * defect correction. Plain BiCGstab stagnates near the critical kappa
   * (SOLVER_BICGSTAB reports that as status 1); this one converges there. */
  QCDGPU_SOLVER_BICGSTABL_EO = 4
};
/* solve A x = b with A = op(g; kappa, mu); x, b FP64 device fields */
int qcdgpu_solve(qcdgpu_field x, qcdgpu_field b, qcdgpu_gauge g, double kappa, double mu,
                 qcdgpu_solve_params *p);

/* Solvers keep their work fields in a pool between calls; this frees the
 * pool's device memory (the next solve allocates again). Returns 0. */
int qcdgpu_release_work(void);
/* Fault injection for tests (no reference counterpart): the next n
 * allocations of host vectors and gauge fields (qcd_initVector,
 * qcd_initGaugeField) and of device fields and gauge fields fail as if memory
 * were exhausted, so that callers' out-of-memory paths run without
 * exhausting memory; n = 0 switches it off. */
int qcdgpu_inject_alloc_failures(int n);
/* Device bytes held by the lazily allocated partial-sum scratch of the
 * reductions (dot products, norms, solver reductions); 0 until the first
 * reduction. Lets a test see that an entry point allocated none. */
int64_t qcdgpu_scratch_bytes(void);
/* FMA throughput of this GPU in TFLOP/s (2 flops per FMA), kind 0 FP64 or 1
 * FP32, from a kernel of independent FMA chains on every SM (no reference
 * counterpart; the benchmark's compute ceilings). */
int qcdgpu_measure_fma_rate(int kind, double *tflops);

/* No counterpart in the reference. The complex dot product
 * result[0] + i result[1] = sum_i conj(a_i) b_i, for callers that cannot
 * allocate device memory (their device heap belongs to a framework's
 * allocator or a pre-reserved serving budget, or they cannot afford the
 * synchronisation an allocation may cause): it allocates nothing. a and b
 * are device arrays of n complex doubles (re, im interleaved, 16-byte
 * aligned), result a device array of 2 doubles; the work is queued on
 * `stream` (a cudaStream_t, NULL = default stream) and the call returns
 * without waiting. Its partial sums live in a fixed 32 KB device array that
 * every call shares: n may not exceed 134,217,728 (larger n returns 1 with a
 * message), and calls that overlap on the GPU race on that array. The first
 * call on each device looks the array's address up; make it before any
 * stream capture. The address stays cached for the process, so the device
 * may not be reset (cudaDeviceReset) while the library is in use. Returns 0,
 * or 1 on error (qcdgpu_last_error). */
int qcdgpu_dot_noalloc(const double *a, const double *b, int64_t n, double *result, void *stream);

/* Source construction on device fields (FP64): n APE steps out <- in (out
 * != in); n Gaussian steps of v on time-slice t; and the smeared point source
 * of the 24^3 x 48 workload: a unit point at x (t, x, y, z), spin, colour,
 * Gaussian-smeared gauss_n times with gauss_alpha on links APE-smeared ape_n
 * times with ape_alpha (on time-slice x[0]). Return 0, or 1 on error. */
/* LIME files straight into / out of device fields (byte order and site
 * order converted on the GPU); source != 0 writes an ETMC source file */
int qcdgpu_gauge_load_lime(qcdgpu_gauge g, const char *fname);
int qcdgpu_gauge_save_lime(qcdgpu_gauge g, const char *fname, const char *message);
int qcdgpu_field_load_lime(qcdgpu_field f, const char *fname);
int qcdgpu_field_save_lime(qcdgpu_field f, const char *fname, int source);
int qcdgpu_gauge_ape3d(qcdgpu_gauge out, qcdgpu_gauge in, double alpha, int n);
int qcdgpu_field_gauss3d(qcdgpu_field v, qcdgpu_gauge g, double alpha, int t, int n);
int qcdgpu_smeared_source(qcdgpu_field f, qcdgpu_gauge g, const int x[4], int spin, int colour, double ape_alpha,
                          int ape_n, double gauss_alpha, int gauss_n);

/* Proton two-point function of twop.c (no qcd_lib library counterpart: the
 * driver twop.c:219-399 computes it inline) on GPU-resident propagators: up
 * and down each 12 FP64 fields, column nu * 3 + c2 = source spin nu, source
 * colour c2 (qcd_lib's D[v][mu][nu][c1][c2]). Source at xsrc (t, x, y, z),
 * theta_t = pi; time-slices t0..t1 relative to the source; mom: nmom
 * momenta (px, py, pz) in units of 2 pi / L. corr[((t - t0) * nmom + j) * 2
 * + {0, 1}] = re, im of the correlator twop.c writes. Returns 0 or 1. */
int qcdgpu_twop_proton(const qcdgpu_field *up, const qcdgpu_field *dn, const int xsrc[4], int t0, int t1,
                       const int *mom, int nmom, double *corr);

/* ---------------------------------------------------------------------- */
/* Multi-RHS (no reference counterpart: qcd_lib solves one column at a time,
 * invert.c:255). A multi-RHS field holds up to 64 spinors in FP16 with one
 * norm per (site, RHS); the operator reads the gauge field once per site
 * for all of them and runs the link x RHS products on the tensor cores. */
typedef struct qcdgpu_mfield_s *qcdgpu_mfield;
int qcdgpu_mfield_create(qcdgpu_mfield *m, const int L[4], int nrhs);
int qcdgpu_mfield_destroy(qcdgpu_mfield m);
/* slot r <- f / f <- slot r (f in any storage precision) */
int qcdgpu_mfield_set(qcdgpu_mfield m, int r, qcdgpu_field f);
int qcdgpu_mfield_get(qcdgpu_field f, qcdgpu_mfield m, int r);
/* out = op(in) for slots 0..nact-1, op QCDGPU_OP_D or QCDGPU_OP_DDAG; g is
 * the FP64 gauge field */
int qcdgpu_dslash_mrhs(qcdgpu_mfield out, qcdgpu_mfield in, qcdgpu_gauge g, double kappa, double mu, int op,
                       int nact);
/* The operator has three kernels: SIMT (one thread per site and RHS, links
 * shared through L1), tcgen05 tensor cores (one FP16 GEMM per site and
 * 16-slot group, the eight hops concatenated along K, FP32 accumulators in
 * tensor memory; slot counts that are multiples of 16) and mma.sync tensor
 * cores (one warp per site, TF32; full lattice only). By default (-1) the
 * first call for a lattice volume and slot count times the SIMT kernel with
 * 64-, 128- and 256-thread blocks and one or two slots per thread and the
 * tensor-core kernels, and keeps the fastest; 1 forces the mma.sync kernel,
 * 2 the tcgen05 kernel, 64 / 128 / 256 (+1: two slots per thread) the SIMT
 * kernel with that block size. */
int qcdgpu_set_mrhs_variant(int variant);
/* the tuned choice for (L, nrhs): variant 0 SIMT / 1 mma.sync / 2 tcgen05
 * and the SIMT block size; returns 1 when nothing has been tuned for it yet */
int qcdgpu_mrhs_tuned(const int L[4], int nrhs, int *variant, int *threads);
/* Every wait of the tcgen05 kernel for its MMAs is bounded. A wait that runs
 * out makes the launch abandon its work (its output is invalid) and sets a
 * failure flag: from then on the multi-RHS operator (qcdgpu_dslash_mrhs and
 * the batches' operator calls), the next chunk boundary of a batch and
 * qcdgpu_sync return 1 with a message, until qcdgpu_mrhs_tc_reset clears the
 * flag. qcdgpu_mrhs_tc_timeouts synchronises the stream and gives *n = the
 * abandoned tiles since the last reset (0 unless the hardware stalled). */
int qcdgpu_mrhs_tc_timeouts(unsigned *n);
int qcdgpu_mrhs_tc_reset(void);
/* Test hook: with skip_mma != 0 the tcgen05 kernel issues no MMA, so its
 * waits run out after `polls` mbarrier polls and the launch reports the
 * timeout; (0, 0) restores normal operation (2^20 polls). */
int qcdgpu_mrhs_tc_test_hook(int skip_mma, int polls);

/* Batched solver with continuous admission (no reference counterpart). A
 * batch of `capacity` slots (1..64) runs mixed-precision CG on the normal
 * equations for every occupied slot at once on the multi-RHS operator, with
 * FP64 reliable updates per slot. Each slot carries its own kappa, mu and
 * tolerance; slots retire when their FP64 true residual |b - op x| / |b|
 * reaches tol and new right-hand sides enter free slots between steps. */
typedef struct qcdgpu_batch_s *qcdgpu_batch;
int qcdgpu_batch_create(qcdgpu_batch *b, qcdgpu_gauge g, int capacity);
/* the same, solving each system through its even/odd Schur complement on
 * the half lattice (every extent even): fewer iterations, same FP64 true
 * residual test; each slot holds one more FP64 half-lattice field (x_e),
 * and keeps two more (c_e, A^{-1} b_o) in its x until it retires */
int qcdgpu_batch_create_eo(qcdgpu_batch *b, qcdgpu_gauge g, int capacity);
int qcdgpu_batch_destroy(qcdgpu_batch b);
/* Solve op x = rhs (op QCDGPU_OP_D or QCDGPU_OP_Q; x, rhs FP64 fields that
 * stay owned by the caller and untouched by it until polled; x holds the
 * slot's work state until then and the solution after; x may be neither the
 * x nor the rhs of another right-hand side in the batch, rhs not another's
 * x). maxiter <= 0: 100000;
 * delta <= 0: 0.1. Returns the slot, -1 when the batch is full, -2 on error.
 * A right-hand side already solved at x_e = 0 (x = 0 for full-lattice
 * batches) is reported by the next poll without taking a slot. */
int qcdgpu_batch_add(qcdgpu_batch b, qcdgpu_field x, qcdgpu_field rhs, double kappa, double mu, int op,
                     double tol, int maxiter, double delta, int tag);
/* Run `iterations` (rounded up to a multiple of 16) iterations of every
 * occupied slot, retiring finished ones. Returns 0 or 3 on a CUDA error. */
int qcdgpu_batch_step(qcdgpu_batch b, int iterations);
int qcdgpu_batch_active(qcdgpu_batch b);
int qcdgpu_batch_free_slots(qcdgpu_batch b);
/* Retired right-hand sides, oldest first: tag, status (0 converged, 1
 * maxiter, 2 breakdown), iterations and true residual. Returns the count. */
int qcdgpu_batch_poll(qcdgpu_batch b, int *tags, int *status, int *iters, double *true_residual, int max);
/* device bytes held by the batch */
size_t qcdgpu_batch_bytes(qcdgpu_batch b);

/* Request server (no reference counterpart): solve requests of different
 * lattices, kappas, twisted masses, RHS counts and tolerances arrive at any
 * time and are served with continuous batching. Each resident gauge field
 * has one batch (qcdgpu_batch) of `slots` slots on its own stream; the
 * batches of different gauge fields run concurrently. A request is admitted
 * (its FP64 solution and source fields allocated) in arrival order when its
 * bytes, and those of its gauge field's batch if that is not yet built, fit
 * in the HBM budget; its right-hand sides enter the batch as slots free up
 * and leave it one by one as they converge. Latencies are wall-clock seconds
 * from submission. */
typedef struct qcdgpu_server_s *qcdgpu_server;
typedef struct {
  int tag;
  int status;               /* 0 all RHS converged, else the worst RHS status */
  int nrhs;
  int max_iters;            /* largest iteration count among the RHS */
  double max_true_residual; /* largest FP64 |b - op x| / |b| among the RHS */
  double queue_s;           /* submission -> admission */
  double latency_s;         /* submission -> last RHS retired */
  int total_iters;          /* iterations summed over the RHS */
} qcdgpu_server_result;
int qcdgpu_server_create(qcdgpu_server *s, size_t hbm_budget_bytes, int slots);
int qcdgpu_server_destroy(qcdgpu_server s);
/* register a resident FP64 gauge field (owned by the caller); returns its
 * id >= 0, or -1 on error */
int qcdgpu_server_add_gauge(qcdgpu_server s, qcdgpu_gauge g);
/* queue a request of nrhs (1..64) right-hand sides on gauge `gauge_id`:
 * op x = b with op QCDGPU_OP_D or QCDGPU_OP_Q. sources: nrhs FP64 fields,
 * copied at admission (they must live until then), or NULL for the
 * spin-colour columns of point sources: column c is spin (c % 12) / 3,
 * colour c % 3 of a point at a position drawn from (seed, c / 12).
 * Returns 0, or 1 on error. */
int qcdgpu_server_submit(qcdgpu_server s, int gauge_id, int nrhs, const qcdgpu_field *sources, uint64_t seed,
                         double kappa, double mu, int op, double tol, int maxiter, int tag);
/* one scheduling step: admission, slot filling; batches (one per gauge
 * field, each on its own stream) run chunks of iterations independently:
 * idle batches with work start a chunk, and the call returns once at least
 * one running chunk has ended (its batch then finished, refilled and
 * relaunched) or at once if none runs. Returns 0, or 3 on a CUDA error. */
int qcdgpu_server_progress(qcdgpu_server s);
/* completed requests, oldest first; returns the count */
int qcdgpu_server_poll(qcdgpu_server s, qcdgpu_server_result *out, int max);
/* copy column `col` of a completed request's solution into dst (FP64) */
int qcdgpu_server_fetch(qcdgpu_server s, int tag, int col, qcdgpu_field dst);
/* free a completed request's fields (and return its bytes to the budget) */
int qcdgpu_server_release(qcdgpu_server s, int tag);
/* bytes held, requests waiting for admission, and admitted RHS not yet
 * retired (in a batch or waiting for a slot) */
int qcdgpu_server_stats(qcdgpu_server s, size_t *bytes_used, int *queued, int *active_rhs);

#ifdef __cplusplus
}
#endif
#endif
