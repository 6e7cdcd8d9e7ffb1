/*
 * sparsesolv_gb300.h -- C ABI of the GB300 (sm_103a) Krylov hot path.
 *
 * This is the boundary the reference's C++ classes and its Python module bind
 * to. Every entry point takes plain pointers and sizes; matrices are CSR with
 * 32-bit indices (slv_int is int in the reference,
 * include/SparseSolv/SparseTypeDefine.hpp:41) and double or interleaved
 * complex-double values (dcomplex = std::complex<double>,
 * include/SparseSolv/BasicDefinesC.hpp:10, which has the same layout).
 *
 * What each entry point replaces in the reference (paths inside SparseSolv):
 *   ssg_create / ssg_destroy     construction of MatSolverICCG / MatSolverMRTR
 *                                (include/SparseSolv/MatSolverICCG.hpp:56-57,
 *                                MatSolverMRTR.hpp:71-72); a handle owns one
 *                                CUDA stream and all device state
 *   ssg_set_options              the setters of MatSolverBase
 *                                (include/SparseSolv/MatSolverBase.hpp:128-137),
 *                                setAccelFactor (MatSolverICCG.hpp:59,
 *                                MatSolverMRTR.hpp:74), setPreconditionType
 *                                (MatSolverMRTR.hpp:75)
 *   ssg_set_matrix[_device]      the SparseMat argument of solve(); CSR taken
 *                                from SparseMatTMPL::getCols/getColPtr/
 *                                getValuePtr (include/SparseSolv/SparseMat.hpp:80-85)
 *   ssg_solve                    MatSolverICCG::solve / MatSolverMRTR::solve,
 *                                pointer overloads with and without normB
 *                                (MatSolverBase.hpp:142-150,
 *                                src/MatSolverICCG.cpp:44-124, :348-424,
 *                                src/MatSolverMRTR_ICver.cpp:44-128, :393-476)
 *   ssg_solve_device             the same solve on device-resident b and x
 *   ssg_solve_multi[_device]     (new) n_rhs right-hand sides in one call, the
 *                                solve(b, x, n_rhs) of the C ABI: solve() once
 *                                per b, sharing the factor and the launches
 *   ssg_get_residual_log         MatSolverBase::getResidualLog
 *                                (src/MatSolverBase.cpp:55-64)
 *   ssg_get_iters                (new) iteration count of the last solve
 *   ssg_factor, ssg_apply_precond, ssg_spmv, ssg_level_schedule
 *                                (new) the hot-path pieces on their own, for
 *                                parity tests and benchmarks:
 *                                SprsPreconditioner::IC_decomp
 *                                (src/SprsPreconditioner.cpp:133-142),
 *                                MatSolverBase::IC_frbc_process
 *                                (src/MatSolverBase.cpp:177-231), Eigen's
 *                                sparse*dense product, and the level schedule
 *                                the GPU sweeps run over
 *   ssg_last_error               (new) message of the last failing call
 *
 * Error behaviour. The reference returns false from solve() when it does not
 * converge, prints "not Convergence!!!", and calls exit(1) when a row of the
 * lower triangle lacks its diagonal (src/SprsPreconditioner.cpp:91-94). Here
 * solve returns SSG_NOT_CONVERGED in the first case and SSG_ERR_NO_DIAGONAL
 * in the second; nothing exits the process. Every device-side wait is bounded
 * and reports SSG_ERR_TIMEOUT instead of hanging.
 *
 * Threading: a handle is not thread-safe (as the reference's solver objects
 * are not); distinct handles may be used from distinct threads.
 */
#ifndef SPARSESOLV_GB300_H
#define SPARSESOLV_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct ssg_handle_s *ssg_handle;

/* return codes */
#define SSG_OK 0
#define SSG_NOT_CONVERGED 1
#define SSG_ERR_ARG (-1)
#define SSG_ERR_CUDA (-2)
#define SSG_ERR_NO_DIAGONAL (-3)
#define SSG_ERR_TIMEOUT (-4)
#define SSG_ERR_NOMEM (-5)
#define SSG_ERR_STATE (-6)

/* solver methods */
#define SSG_METHOD_ICCG 0 /* MatSolverICCG: shifted ICCG (real) / ICCOCG (complex) */
#define SSG_METHOD_MRTR 1 /* MatSolverMRTR: precondition_type 0 = IC, 1 = Eisenstat SGS */

/* value types */
#define SSG_REAL 0    /* double */
#define SSG_COMPLEX 1 /* interleaved (re, im) doubles, unconjugated bilinear products */

/* precision modes (build addition; does not change the method) */
#define SSG_PREC_FP64 0  /* everything in FP64, as the reference */
#define SSG_PREC_MIXED 1 /* FP32 factor, SpMV and sweeps inside an inner loop,
                            FP64 outer residual and iterative refinement: the IC factor
                            and its shift are computed in FP64 and rounded; each inner
                            ICCG / IC-MRTR (FP32 vectors, FP64 scalars) reduces the
                            scaled residual r/|r| by 1e-4 (real) or 1e-2 (complex), or
                            ends after 30 iterations without a 1% gain (FP32 rounding
                            bounds what one inner solve can reach); x += |r| d and r = b - A x
                            run in FP64 until |b - A x| / |b| < conv_cri (a true
                            residual). ssg_solve: ICCG or IC-MRTR, accel_factor > 0,
                            is_init = 1, conv_normalize_type 0, no diagonal scaling;
                            iterations count inner iterations, the residual log holds
                            |b - A x| / |b| after each refinement step. */

/*
 * Settings with the reference's defaults (src/MatSolverBase.cpp:32-47,
 * include/SparseSolv/MatSolverICCG.hpp:40, MatSolverMRTR.hpp:40-43).
 * Fill with ssg_default_options().
 */
typedef struct {
    int is_init;              /* 1: start from x = 0 (setInitSolution) */
    int is_diag_scale;        /* setDiagScale */
    int is_save_best;         /* setSaveBest */
    int is_save_residual_log; /* setSaveLog */
    int diverge_judge_type;   /* setDirvegeType: 0 none, 1 bad-count judge */
    double bad_div_val;       /* setBadDivVal */
    int bad_div_count_thres;  /* setBadDivCount */
    int conv_normalize_type;  /* setConvNormalizeType: 0 |b|, 1 |r0|, 2 const */
    double conv_normalize_const; /* setConvNormalizeConst */
    double accel_factor;      /* setAccelFactor (alpha < 0: automatic search) */
    int precondition_type;    /* setPreconditionType (MRTR): 0 IC, 1 SGS */
    int precision;            /* SSG_PREC_* */
    int mrtr_reference_quirks;/* 1: reproduce the reference's IC-MRTR p update and
                                 MRTR warm start (default 0: corrected) */
} ssg_options;

void ssg_default_options(ssg_options *o);

int ssg_create(ssg_handle *h, int device);
int ssg_destroy(ssg_handle h);
const char *ssg_last_error(ssg_handle h);
int ssg_set_options(ssg_handle h, const ssg_options *o);

/* CSR from host memory; values are double[nnz] or (re,im) double[2*nnz] */
int ssg_set_matrix(ssg_handle h, int n, int nnz, const int32_t *row_ptr, const int32_t *col,
                   const double *val, int value_type);
/* CSR already in device memory (copied device to device) */
int ssg_set_matrix_device(ssg_handle h, int n, int nnz, const int32_t *d_row_ptr, const int32_t *d_col,
                          const double *d_val, int value_type);
/* The matrix from COO triplets (row, col, value), built on the device: the
 * counterpart of SparseBuilder::build + SparseMat(builder, to_square = true)
 * (src/SparseBuilder.cpp:107-141, src/SparseMat.cpp:114-122) and of the COO
 * constructor (src/SparseMat.cpp:80-104). n x n, columns ascending within a
 * row, a (row, col) given several times summed in input order, as
 * Eigen::setFromTriplets does; an entry outside [0, n) returns SSG_ERR_ARG.
 * rows/cols/vals in host memory, or device memory with on_device = 1. */
int ssg_set_matrix_coo(ssg_handle h, int n, int nnz, const int32_t *rows, const int32_t *cols, const double *vals,
                       int value_type, int on_device);
/* copy of the current matrix as CSR (host buffers; null pointers skip; n and nnz report the sizes) */
int ssg_get_matrix(ssg_handle h, int32_t *row_ptr, int32_t *col, double *val, int *n, int *nnz);
/* Post-processing: flux density B = curl A at the centre of every voxel of an
 * nx x ny x nz grid of hx x hy x hz elements, from the edge unknowns A[nunk]
 * of a solution (real, or complex for eddy-current systems); the counterpart of
 * Element::calcB of the reference's VoxelFEM example (examples/VoxelFEM/
 * Element.cpp:116-168). ex/ey/ez[(nx+1)(ny+1)(nz+1)]: unknown of the x/y/z edge
 * starting at node x + (nx+1)(y + (ny+1) z), -1 where there is none (Dirichlet);
 * B[3 * (x + nx (y + ny z)) + c]. Host buffers, or device with on_device = 1. */
int ssg_flux_density(ssg_handle h, int nx, int ny, int nz, double hx, double hy, double hz, const int32_t *ex,
                     const int32_t *ey, const int32_t *ez, int nunk, const void *A, int value_type, void *B,
                     int on_device);

/* The voxel edge-element system assembled on the device straight into the
 * handle's matrix, with its T-method right-hand side: the system of the
 * reference's VoxelFEM example (examples/VoxelFEM/VoxelMatrix.cpp:118-201,
 * :24-114), which the example builds on the host through SparseBuilder; no
 * counterpart in the library itself. Bit-identical to the host generator
 * (sparsesolv_gb300/voxel/voxelgen.c):
 *   K_rc = sum over the elements e holding edges r and c, in ascending element
 *          index, of nu[e] Ke[k][m] (+ j sig[e] omega Me[k][m] when complex),
 *   b_r  = sum over the elements holding r of sum_{m = 8..11, tz != 0} Ce[k][m] tz_m,
 * each product and sum rounded on its own; columns ascending, explicit zeros kept.
 * nx, ny, nz voxels; ex/ey/ez[(nx+1)(ny+1)(nz+1)]: unknown of the x/y/z edge
 * starting at node x + (nx+1)(y + (ny+1) z), -1 where there is none; nunk
 * unknowns; Ke/Me/Ce: the 12 x 12 element matrices (row-major, local edge
 * l = 4 d + 2 b + a, always host memory); nu[nx ny nz] per element
 * (x + nx (y + ny z)); sig (may be null), omega; tz[(nx+1)(ny+1) nz] the line
 * integral of T on the z-edge starting at node x + (nx+1)(y + (ny+1) z) (may be
 * null: b = 0). value_type SSG_REAL or SSG_COMPLEX; b (may be null) receives
 * nunk values of that type. ex..tz and b in host memory, or device memory with
 * on_device = 1. Maps that do not match nunk return SSG_ERR_ARG. */
int ssg_set_matrix_voxel(ssg_handle h, int nx, int ny, int nz, const int32_t *ex, const int32_t *ey,
                         const int32_t *ez, int nunk, const double *Ke, const double *Me, const double *Ce,
                         const double *nu, const double *sig, double omega, const double *tz, int value_type, void *b,
                         int on_device);

/*
 * One solve() call. b and x are host arrays of n values (x is in/out: the
 * initial guess when is_init = 0, the solution on return). normB < 0 makes
 * the solver compute |b| itself (the overloads without normB). Returns
 * SSG_OK (converged), SSG_NOT_CONVERGED, or an error code.
 */
int ssg_solve(ssg_handle h, int method, double conv_cri, int max_ite, double normB, const double *b, double *x);
int ssg_solve_device(ssg_handle h, int method, double conv_cri, int max_ite, double normB, const double *d_b,
                     double *d_x);
/*
 * Several right-hand sides of the handle's matrix in one call (the C ABI's
 * solve(b, x, n_rhs); the reference solves one b per solve() call,
 * src/MatSolverICCG.cpp:44-124, src/MatSolverMRTR_ICver.cpp:44-128). B and X hold
 * n_rhs vectors of n values one after another (X in/out as in ssg_solve); iters and
 * status (may be NULL) receive per right-hand side the iteration count and SSG_OK /
 * SSG_NOT_CONVERGED. Returns SSG_OK when every right-hand side converged.
 * With the settings of a batch (ICCG or IC-MRTR, fixed accel_factor > 0, is_init = 1,
 * conv_normalize_type 0, no diagonal scaling, no save-best, no divergence judge) and
 * n_rhs > 1, the right-hand sides share one factor and run in the same launches: each
 * is solved as its own batch instance (the same method and stopping rule; numbers
 * agree with ssg_solve to rounding). Otherwise they are solved one after another
 * exactly as ssg_solve solves them.
 * The residual log afterwards is that of the last right-hand side.
 */
int ssg_solve_multi(ssg_handle h, int method, double conv_cri, int max_ite, int n_rhs, const double *B, double *X,
                    int *iters, int *status);
int ssg_solve_multi_device(ssg_handle h, int method, double conv_cri, int max_ite, int n_rhs, const double *d_B,
                           double *d_X, int *iters, int *status);

/* new values for the current pattern (same n, nnz, row_ptr, col); invalidates the factor */
int ssg_update_values(ssg_handle h, const double *val);
int ssg_update_values_device(ssg_handle h, const double *d_val);

int ssg_get_residual_log(ssg_handle h, double *log, int cap, int *len);
int ssg_get_iters(ssg_handle h, int *iters);
/* accel factor actually used by the last factorisation (after an automatic search) */
int ssg_get_accel_used(ssg_handle h, double *alpha);
/* time of the phases of the last solve, milliseconds: [0] setup+factor, [1] iterations */
int ssg_get_timings(ssg_handle h, double *ms, int cap);

/* ---- measurement (new) ---- */
/* the CUDA stream all work of the handle runs on (a cudaStream_t) */
int ssg_get_stream(ssg_handle h, void **stream);
/* per-kernel-class CUDA-event timing of the following solves (0 off, 1 on) */
int ssg_set_profiling(ssg_handle h, int enable);
/* classes: 0 forward sweep, 1 backward sweep, 2 SpMV, 3 fused vector/reduction
 * kernels, 4 IC factor, 5 level schedule; per class the summed device time
 * (ms), the launch count and the algorithmic bytes moved (unit model of each
 * kernel); accumulated since the last ssg_set_profiling(h, 1) */
int ssg_get_kernel_stats(ssg_handle h, double *ms, long long *launches, double *bytes, int cap);
/* kernels this library has launched in the process so far */
long long ssg_launch_count(void);

/* launch tuning (new; results do not depend on it beyond last-bit rounding) */
#define SSG_TUNE_SWEEP_CTA_PER_SM 0  /* resident CTAs per SM claiming sweep rows (0, default: from the mean
                                        level width, 2 for levels of about a thousand rows, up to 16) */
#define SSG_TUNE_SWEEP_GROUP 1       /* lanes per row in the sweeps: 0 auto, 4, 8, 16, 32 */
#define SSG_TUNE_SWEEP_BACKOFF_NS 2  /* sleep between polls of an unsolved entry */
#define SSG_TUNE_FACTOR_BACKOFF_NS 3 /* sleep between polls of an unfinished factor row */
#define SSG_TUNE_RECIPROCAL_DIAG 4   /* 1 (default): multiply by precomputed 1/diagonal in the sweeps */
#define SSG_TUNE_SWEEP_MODE 5        /* 0 auto (default: for real values the push sweep, else the one-cluster
                                        sweep, where their plans fit), 1 sync-free, 2 one-cluster level-synchronous,
                                        3 one-cluster neighbour-synchronised (IC sweeps; others as 2), 4 one-cluster
                                        push: no cluster-wide barrier, each value pushed to the CTAs that read it,
                                        rows summed in dependency-level order (IC sweeps; others as 2) */
#define SSG_TUNE_CLUSTER_RING_KB 6   /* distributed shared-memory ring per CTA of the cluster sweep (KB) */
#define SSG_TUNE_CLUSTER_GROUP 7     /* lanes per row in the cluster sweep: 4 (default), 8, 16, 32 */
#define SSG_TUNE_SPMV_GROUP 9        /* lanes per row in the SpMV: 0 (default: about 8 entries a lane for real
                                        rows, 16 for complex: 4 and 2 lanes for the voxel systems), 2, 4, 8, 16, 32 */
#define SSG_TUNE_BATCH_GROUP 8       /* lanes per row in both sweeps of the handle's internal batch (ssg_solve_multi,
                                        mixed precision): 0 (default: 4 for one real right-hand side, 8 for one
                                        complex one; for several,
                                        16 when the lower rows hold more than 6 off-diagonal entries on average,
                                        else 8), 4, 8, 16; the internal batch also follows SSG_TUNE_SWEEP_MODE
                                        and SSG_TUNE_SWEEP_CTA_PER_SM */
#define SSG_TUNE_SPIN_LIMIT_US 10    /* how long a bounded device wait (factor row flags, sync-free sweep values,
                                        level schedule, neighbour-synchronised progress) polls before it gives up
                                        and the call returns SSG_ERR_TIMEOUT, in microseconds; 0 (default): 4 s.
                                        A short limit makes waits that would have succeeded fail: for tests of the
                                        timeout path; the handle stays usable after such a failure */
int ssg_set_tuning(ssg_handle h, int key, int value);
/* Autotuner (build addition): times the IC preconditioner of the current matrix
 * and factor for each candidate sweep schedule (sync-free with 4/8/16 lanes a row
 * and 2/4/8/16/automatic CTAs per SM; one-cluster level-synchronous and
 * neighbour-synchronised with 4/8 lanes), keeps the fastest in the handle's
 * tuning and reports it. keep_group = 1 keeps the current lanes per row, so
 * results stay bit-identical to an untuned run; otherwise they may change at
 * rounding level (a row's entries are summed in another order). */
int ssg_autotune(ssg_handle h, int keep_group, int *mode, int *group, int *cta_per_sm, double *ms);

/* ---- hot-path pieces on their own (host buffers) ---- */
/* IC(0) factor of the current matrix with shift alpha: L in the lower(A) pattern
 * (lrp[n+1], lci[nnzL], lval[nnzL] values) and D = 1/pivot (n values). */
int ssg_factor(ssg_handle h, double alpha, int32_t *lrp, int32_t *lci, double *lval, double *D, int *nnzL);
/* z = (L D L^T)^{-1} r with the factor of the last ssg_factor call */
int ssg_apply_precond(ssg_handle h, const double *r, double *z);
/* y = A x */
int ssg_spmv(ssg_handle h, const double *x, double *y);
/* level schedule of the lower (lower = 1) or upper (lower = 0) triangle of the
 * current matrix: level[n], perm[n] (rows by level, then row id), returns the
 * number of levels in *nlev */
int ssg_level_schedule(ssg_handle h, int lower, int32_t *level, int32_t *perm, int *nlev);

/* ---- batches: many systems in shared launches (no counterpart in the reference) ----
 * Independent systems of uneven sizes, each with one or more right-hand
 * sides, solved together. Every (system, right-hand side) pair is an instance;
 * the instances are concatenated into one block-diagonal matrix, so one
 * launch of each kernel serves all of them, while every instance keeps its
 * own Krylov scalars, convergence test and iteration count, as if it had been
 * solved alone by MatSolverICCG / MatSolverMRTR (IC preconditioner) with x0 = 0,
 * a fixed shift alpha, conv_normalize_type 0 and no diagonal scaling. An
 * instance's results do not depend on the other instances of its batch.
 * The systems of one batch are all real or all complex. A right-hand side of a
 * system is stored as its own instance (the matrix is repeated per
 * right-hand side). Host buffers; X and B hold n_rhs vectors of n values
 * one after another (interleaved re, im for SSG_COMPLEX). */
typedef struct ssg_batch_s *ssg_batch;
int ssg_batch_create(ssg_batch *out, int device);
int ssg_batch_destroy(ssg_batch b);
const char *ssg_batch_last_error(ssg_batch b);
/* adds a system (CSR as for ssg_set_matrix) and its right-hand sides; *index numbers it */
int ssg_batch_add(ssg_batch b, int n, int nnz, const int32_t *row_ptr, const int32_t *col, const void *val,
                  int value_type, int n_rhs, const void *B, int *index);
/* replaces the n_rhs right-hand sides of system `index` for the next start (the others stay on the device) */
int ssg_batch_set_rhs(ssg_batch b, int index, const void *B);
int ssg_batch_clear(ssg_batch b);
/* uploads the systems (first start after add/clear), factors every system with
 * shift alpha and queues the first iterations; returns without waiting */
int ssg_batch_start(ssg_batch b, int method, double alpha, double conv, int max_ite);
/* non-blocking: queues further iterations when the previous ones finished; *done = 1 once every instance ended */
int ssg_batch_poll(ssg_batch b, int *done);
int ssg_batch_wait(ssg_batch b);
/* blocking for the iterations in flight only, then as ssg_batch_poll */
int ssg_batch_step(ssg_batch b, int *done);
/* *finished = 1 once every right-hand side of system `index` ended, as of the last
 * completed iterations; its ssg_batch_result is then available while the batch runs on */
int ssg_batch_finished(ssg_batch b, int index, int *finished);
/* solution, iteration counts and statuses (ST_* : 1 converged, 2 max_ite, 3 diverged) of system `index`,
 * after the batch ended or once ssg_batch_finished reports the system;
 * returns SSG_OK when all its right-hand sides converged, else SSG_NOT_CONVERGED */
int ssg_batch_result(ssg_batch b, int index, void *X, int *iters, int *status);
int ssg_batch_residual_log(ssg_batch b, int index, int rhs, double *log, int capacity, int *length);
/* set-up and iteration time of the last solve (ms, CUDA events) */
int ssg_batch_timings(ssg_batch b, double *ms2);
/* SSG_PREC_FP64 (default) or SSG_PREC_MIXED (see above) for the next start; inner_tol <= 0: 1e-4 real, 1e-2 complex */
int ssg_batch_set_precision(ssg_batch b, int precision, double inner_tol);
int ssg_batch_stream(ssg_batch b, void **stream);
/* per-kernel-class event timing of the batch's solves, as ssg_set_profiling / ssg_get_kernel_stats */
int ssg_batch_set_profiling(ssg_batch b, int enable);
/* 1 (default): each start captures 8 iterations in a CUDA graph once and replays it
 * for the later chunks (direct launches while profiling); 0: direct launches only */
int ssg_batch_set_graphs(ssg_batch b, int enable);
/* 1 (default): FP64 ICCG starts run persistent: one CTA per (system, right-hand side) runs all
 * of its iterations (SpMV, update and convergence test, both IC sweeps level by level
 * with a CTA barrier between levels, beta, p) with no further launch and no wait on
 * another CTA; the same bits as the launch-per-phase iterations with the sync-free
 * sweep. Used when every system has at most 16,384 rows, the sweeps have a fixed lane
 * count (the batch default, 8) and the reciprocal diagonal is on; otherwise, and for
 * IC-MRTR and mixed precision, the launches run. 0: launches always. On 1,024
 * instances of 1-4k rows: 24,300 solves/s against 19,600 with the launches. No
 * reference counterpart (the reference solves one system per call). */
int ssg_batch_set_persistent(ssg_batch b, int enable);
/* Times the sweep schedules on the batch's block-diagonal matrix (as ssg_autotune:
 * sync-free with 4/8/16 lanes a row and 2..16 CTAs per SM, one-cluster lockstep and
 * neighbour-synchronised with 4/8) and keeps the fastest for the following starts.
 * Results stay deterministic; an instance's bits then follow the lanes a row chosen
 * for this batch instead of the fixed 8 (the same instance in another batch may
 * differ at rounding level). Assembles the batch if needed; not while it runs. */
int ssg_batch_autotune(ssg_batch b, int *mode, int *group, int *cta_per_sm, double *ms);
int ssg_batch_kernel_stats(ssg_batch b, double *ms, long long *launches, double *bytes, int capacity);

/* ---- IC(0) factor that allocates nothing (no counterpart in the reference) ----
 * For callers that may not call cudaMalloc: code that runs under an external
 * memory manager which owns all device memory, or a real-time loop where an
 * allocation's latency or failure is not allowed. Unlike ssg_create/
 * ssg_set_matrix/ssg_factor it needs no handle and allocates no memory, host or
 * device: its scratch (one flag per row, a row ticket, an error word) is a
 * file-scope array of the library, (64 + SSG_NOALLOC_MAX_ROWS) ints = 8 MB, that
 * every GPU which loads the library holds until the process exits.
 *
 * All pointers are device memory on the calling thread's current device:
 *   lrp[n+1], lci[nnz]  lower triangle of A including the diagonal, CSR in
 *                       natural row order, columns strictly ascending, diagonal
 *                       last in each row, at most 32 entries a row (the pattern
 *                       ssg_factor returns); 4-byte aligned
 *   lower_val[nnz]      A's values on that pattern (double, 8-byte aligned, or
 *                       interleaved complex, 16-byte aligned, for value_type
 *                       SSG_COMPLEX; lval and D have the same alignment)
 *   lval[nnz], D[n]     outputs: L on the same pattern and D = 1/pivot, the
 *                       shifted IC(0) of src/SprsPreconditioner.cpp:43-111;
 *                       lval may be lower_val (factor in place)
 *   alpha > 0           the shift (acceleration factor); no automatic search
 * Work is queued on `stream` (NULL: the legacy default stream) and the call
 * waits for it, so the result is ready on return. Returns SSG_OK,
 * SSG_ERR_ARG (n > SSG_NOALLOC_MAX_ROWS, a null or misaligned pointer, a row
 * longer than 32 entries, a column out of range or columns not ascending),
 * SSG_ERR_NO_DIAGONAL, SSG_ERR_TIMEOUT or SSG_ERR_CUDA; every argument check
 * is made before any GPU work. A stream that is capturing work into a CUDA
 * graph is refused with SSG_ERR_STATE before anything is queued: the call
 * reads its status back to the host and waits. The first call on a device
 * looks up the array's device address (once per device, cudaGetSymbolAddress).
 * All calls share the one array and it keeps the last call's contents (each
 * call clears what it uses), so calls whose work overlaps on the GPU (other
 * threads, other streams) race: serialise them. A call that fails after its
 * kernel was queued waits for that kernel before it returns, so the array is
 * idle whenever a call has returned. */
#define SSG_NOALLOC_MAX_ROWS (1 << 21)
int ssg_ic_factor_noalloc(int n, int nnz, const int32_t *lrp, const int32_t *lci, const void *lower_val, void *lval,
                          void *D, double alpha, int value_type, void *stream);

#ifdef __cplusplus
}
#endif

#endif
