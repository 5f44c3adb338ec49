/*
 * kore_gpu.h — C ABI of libkoregpu.so, the GB300 (sm_103a) solve path of kore.
 *
 * The reference solve path is the script bin/solve.py, which has no in-process API:
 * it reads A.npz / B.npz (or B_forced.npz), builds PETSc matrices and hands them to
 * SLEPc (eigenproblem) or a KSP direct solve (forced problem).  Each entry point
 * below replaces one step of that script; the Python host (kore_gb300.solver and the
 * drop-in kore_gb300/cli/solve.py) binds them with ctypes.
 *
 * Conventions
 *  - Every function returns an int status (KORE_OK = 0 or a KORE_E* code).
 *  - Complex numbers are interleaved (re, im) doubles, i.e. numpy complex128.
 *  - All matrix and vector arguments are HOST pointers unless the name ends in _dev,
 *    in which case they are device pointers on the plan's device and the call is
 *    asynchronous on the given CUDA stream (0 = the plan's stream).
 *  - Vectors are in the ORIGINAL (section-major) unknown order of bin/assemble.py;
 *    the l-major permutation is internal to the plan.
 *  - A plan is used by one host thread at a time; distinct plans are independent.
 */
#ifndef KORE_GPU_H
#define KORE_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define KORE_OK          0
#define KORE_EINVAL      1   /* bad argument or a matrix entry outside the block-tridiagonal band */
#define KORE_ENOMEM      2   /* device allocation failed */
#define KORE_ECUDA       3   /* a CUDA runtime error */
#define KORE_ESINGULAR   4   /* zero pivot in a diagonal Schur complement */
#define KORE_ENOCONV     5   /* eigensolver: nothing converged within maxit restarts */
#define KORE_ETIMEOUT    6   /* a bounded device wait ran out (error flag set by a kernel) */
#define KORE_ENOTFACTORED 7  /* solve/eigs before kore_factor */
#define KORE_ENAN        8   /* NaN or Inf in a solution (bin/solve.py:263-268) */
#define KORE_EPENDING    9   /* kore_batch_poll: the request has not finished yet */
#define KORE_ECANCELLED 10   /* kore_batch_destroy dropped the request before it started */

/* factorisation precisions */
#define KORE_PREC_FP64   0   /* complex128 block LU, complex128 sweeps */
#define KORE_PREC_MIXED  1   /* complex64 block LU, FP64 iterative refinement */

/* SLEPc 'which' criteria, same order as bin/solve.py:99-117 */
#define KORE_WHICH_LM 0
#define KORE_WHICH_SM 1
#define KORE_WHICH_LR 2
#define KORE_WHICH_SR 3
#define KORE_WHICH_LI 4
#define KORE_WHICH_SI 5
#define KORE_WHICH_TM 6
#define KORE_WHICH_TR 7
#define KORE_WHICH_TI 8

typedef struct kore_plan kore_plan;

/*
 * The pencil (A, B) in the CSR form bin/assemble.py writes with np.savez
 * (bin/assemble.py:591 for B, :1171 for A; loaded by bin/utils.py:1253-1256).
 * A is complex128, B is float64; B may be absent (b_nnz = 0, pointers NULL) for the
 * forced problem.  perm[i] is the original index of l-major unknown i; block_sizes
 * partitions the l-major order into nblocks consecutive diagonal blocks such that
 * A and B are block tridiagonal.  The plan copies everything it needs; the caller's
 * arrays may be freed after the call.
 */
typedef struct {
    int64_t n;
    int64_t a_nnz;
    const int32_t *a_indptr;    /* n + 1 */
    const int32_t *a_indices;   /* a_nnz */
    const double  *a_data;      /* 2 * a_nnz (re, im) */
    int64_t b_nnz;
    const int32_t *b_indptr;    /* n + 1, or NULL */
    const int32_t *b_indices;   /* b_nnz, or NULL */
    const double  *b_data;      /* b_nnz, or NULL */
    const int64_t *perm;        /* n */
    int32_t nblocks;
    const int32_t *block_sizes; /* nblocks */
} kore_pencil_desc;

/*
 * Krylov-Schur options: the fields bin/solve.py sets on SLEPc EPS
 * (setDimensions(nev) :96, setTolerances(tol, maxit) :97, setWhichEigenpairs :99-117,
 * setTarget(tau) :119) plus the explicit dimensions SLEPc would choose
 * (ncv = 0 -> min(n, max(2 nev, nev + 15, min(64, 4 nev))): SLEPc's default raised
 * to 4 nev, up to 64, because on the GPU a larger basis saves more operator
 * applications than it costs).
 */
typedef struct {
    int32_t nev;
    int32_t ncv;          /* 0 = default (see above) */
    double  tol;          /* relative, on the transformed eigenvalue theta */
    int32_t maxit;        /* restarts */
    int32_t which;        /* KORE_WHICH_TM, _TR or _TI: shift-and-invert needs a target
                             criterion (SLEPc refuses the others under sinvert) */
    double  target_re, target_im;   /* tau: `which` measures distances from it */
    uint64_t seed;        /* start vector: complex standard normal from this seed */
    int32_t purify;       /* applications of OP to each eigenvector before it is
                             returned: 1 is SLEPc's default purification, 0 none */
    double  refine_tol;   /* mixed precision: relative residual of each OP application
                             (<= 0 selects 1e-16); the purifying application of the
                             eigenvectors is refined until the residual stops decreasing */
    /* Spectral-transformation shift sigma (SLEPc's -st_shift): OP = (A - sigma B)^-1 B and
     * lambda = sigma + 1/theta, while `which` still measures from the target.  has_shift = 0:
     * sigma is the target (SLEPc's default).  The factorised shift must equal sigma. */
    double  shift_re, shift_im;
    int32_t has_shift;
    /* 1: start from the normalised sum of the eigenvectors the previous target in the same
     * slot returned (the plan keeps one such vector per slot), when there is one, instead
     * of the seeded vector.  The result then depends on that earlier solve. */
    int32_t warm;
    /* Batched and served eigensolves (kore_eigs_shifts, the serving queue): > 0 lets a target
     * run on an idle slot whose factorised shift lies within this distance of the target,
     * as sigma of that slot, without re-factorising.  0: only a slot holding exactly the
     * target's shift is reused. */
    double  reuse_radius;
} kore_eps_opts;

/* Per-call statistics, filled by kore_eigs / kore_solve when the pointer is non-NULL. */
typedef struct {
    int32_t nconv;
    int32_t restarts;          /* Krylov-Schur outer iterations */
    int32_t op_applies;        /* applications of (A - sigma B)^-1 B */
    int32_t sweeps;            /* block-tridiagonal forward+back sweeps */
    int32_t refine_iters_max;  /* mixed precision: worst refinement count of one application */
    double  solve_resid_max;   /* worst relative residual of one application */
    double  factor_ms, iterate_ms;
    int32_t factor_reused;     /* eigen: the slot already held the factors of the shift used */
    int32_t warm_started;      /* eigen: started from the slot's last eigenvectors (opts.warm) */
    double  shift_re, shift_im;   /* eigen: the shift of the spectral transformation used */
    int32_t escalated;         /* served forced request: solved again with FP64 factors because the
                                  mixed refinement stopped above 1e-10 */
} kore_stats;

/* Replaces bin/solve.py:40-86 (load_csr + PETSc Mat assembly of A and B). */
int kore_plan_create(const kore_pencil_desc *desc, int device, kore_plan **plan);

/*
 * Factorises A - sigma B (block cyclic reduction over the l-major blocks: explicit
 * inverses of the eliminated diagonal blocks by Gauss-Jordan with partial pivoting,
 * their couplings G = D^-1 L, H = D^-1 U, Schur-complement updates of the surviving
 * blocks, level by level).  Replaces the LU that SLEPc's ST sinvert builds inside E.solve()
 * (bin/solve.py:123) and the KSP preonly+LU factorisation (bin/solve.py:220-227).
 */
int kore_factor(kore_plan *plan, double sigma_re, double sigma_im, int precision);

/*
 * Factorises A - sigma_s B for nshift shifts at once (sigmas: nshift interleaved
 * re, im pairs), e.g. the forcing frequencies sigma = i*omega of a batch of forced
 * problems on one eigen pencil (bin/assemble.py makes the forced matrix
 * ||u||_F (A_eig - i omega B_eig)).  Every kernel of the factorisation and of the
 * solves covers all shifts in one launch.  kore_factor is the nshift = 1 case.
 */
int kore_factor_shifts(kore_plan *plan, int nshift, const double *sigmas, int precision);

/*
 * x = (A - sigma B)^-1 b for nrhs right-hand sides stored one after another
 * (column k at b + 2*n*k); with several factorised shifts nrhs must be a multiple of
 * nshift and right-hand side k is solved with shift k % nshift.  Replaces
 * K.solve(bvec, x) (bin/solve.py:227).  In mixed precision the result is refined in
 * FP64 to relative residual <= refine_tol (refine_tol <= 0 selects 1e-14).
 */
int kore_solve(kore_plan *plan, const double *b, double *x, int nrhs, double refine_tol,
               kore_stats *stats);
int kore_solve_dev(kore_plan *plan, const void *b_dev, void *x_dev, int nrhs,
                   double refine_tol, void *stream, kore_stats *stats);

/*
 * x = (A - sigma B)^-1 b for one right-hand side, like kore_solve_dev, but without
 * allocating anything: no cudaMalloc/cudaFree and no allocating library routine.
 * This entry point has no counterpart in the reference; it is for callers that
 * cannot allocate device memory when they solve (a fixed memory budget or a pool they
 * do not own, a latency-critical loop that must not take the device-wide
 * synchronisation of cudaMalloc/cudaFree, a host library handed only a stream).
 * Its scratch is one file-scope device array of fixed size held by every GPU that
 * loads the library until exit; problems with more than 16384 padded unknowns
 * (blocks x largest block size) are rejected with KORE_EINVAL and a message on
 * stderr.  The plan must hold one factorised shift (kore_factor); a plan of several
 * shifts (kore_factor_shifts) is rejected with KORE_EINVAL.  b_dev and x_dev are
 * complex128 device vectors in the original unknown order; the kernels run on
 * `stream` (0 = the legacy default stream) of the plan's device, and before returning
 * the call synchronises that stream and copies the scratch's error and NaN flags to
 * the host (KORE_ETIMEOUT, KORE_ENAN), so no call can be part of a stream capture
 * (a call made while its stream captures invalidates the capture and returns
 * KORE_ECUDA).  The first call on a device looks up the scratch address.  Every
 * call shares the one scratch array and keeps the last call's contents, so calls
 * whose work overlaps on the GPU (other threads, other streams) race: serialise them.
 */
int kore_solve_dev_noalloc(kore_plan *plan, const void *b_dev, void *x_dev, double refine_tol,
                           void *stream);

/*
 * Shift-and-invert Krylov-Schur for A x = lambda B x around the factorised shift
 * (one shift: KORE_EINVAL after kore_factor_shifts with nshift > 1).
 * Replaces E.solve() and the getEigenpair loop (bin/solve.py:123-158).  evals
 * receives up to ncv complex eigenvalues in SLEPc order (converged first, sorted by
 * `which`), evecs (may be NULL) up to ncv unit-2-norm eigenvectors in the original
 * unknown order; *nconv is the number of converged pairs.  Capacity of evals/evecs:
 * max_pairs pairs.
 */
int kore_eigs(kore_plan *plan, const kore_eps_opts *opts, double *evals, double *evecs,
              int max_pairs, int *nconv, kore_stats *stats);

/*
 * Batched form of kore_eigs with continuous admission: ntarget independent
 * shift-and-invert Krylov-Schur solves on one pencil, run in the plan's nshift
 * factorised shifts as slots (kore_factor_shifts, nshift <= 32).  Targets 0 .. nshift-1
 * must be the factorised shifts (opts[t].target = shift t); when a target finishes, the
 * next one (targets nshift .. ntarget-1) takes its slot: the slot alone is re-factorised
 * at opts[t].target, in the plan's precision, while the other slots carry on.  Each
 * target has its own options opts[t] (nev, ncv, tol, maxit, which, seed, purify; the
 * refinement tolerance of opts[0] applies to all).  The busy slots step together: each
 * step applies OP once for every busy slot in shared launches (one sparse product and
 * one sweep over all shifts), and each target's results are those of kore_eigs at that
 * target.  Target t writes evals + 2 * max_pairs * t, evecs + 2 * n * max_pairs * t (may
 * be NULL), nconv[t] and stats[t] (may be NULL).  Returns KORE_ENOCONV when a target
 * converged no pair.  The reference runs one bin/solve.py process per target
 * (bin/solve.py:91-158, driven over parameter sweeps by tools/dodirs.sh); this replaces
 * that fan-out.
 */
int kore_eigs_shifts(kore_plan *plan, int ntarget, const kore_eps_opts *opts, double *evals, double *evecs,
                     int max_pairs, int *nconv, kore_stats *stats);

/* y = A x - lambda B x (FP64, original order, host pointers); residual checks. */
int kore_residual(kore_plan *plan, double lam_re, double lam_im, const double *x, double *y);

/*
 * Pins the sweep variant for every later sweep of the process: ctas_per_sm 2, 3 or 4
 * and chunk_bytes 8192 or 16384 (the ring slot size); (0, 0) restores the autotuner,
 * which otherwise times the six variants on the first sweep of each plan shape and
 * keeps the fastest.  KORE_EINVAL for any other pair.  For reproducible timings and
 * for testing each variant.
 */
int kore_sweep_variant(int ctas_per_sm, int chunk_bytes);

/* The CUDA stream (cudaStream_t) every kernel of the plan is launched on. */
int kore_plan_stream(const kore_plan *plan, void **stream);

/*
 * Kernel timing with CUDA events on the plan's stream.  enable = 1 starts recording
 * (and clears the totals), 0 stops.  out (may be NULL) receives 14 doubles:
 * [sweep kernel ms total, sweeps that ran, factorisation ms total, factorisations,
 *  algorithmic bytes of one sweep launch, algorithmic flops of one factorisation,
 *  sparse-product ms, count, orthogonalisation ms, count, projected-problem ms, count,
 *  CTAs per SM and ring chunk bytes of the last sweep launch].
 */
int kore_profile(kore_plan *plan, int enable, double *out);

/* Device bytes held by the plan (CSR copies + factors + Krylov workspace). */
int kore_plan_bytes(const kore_plan *plan, int64_t *bytes);

/*
 * Upper bound of the device bytes a plan of this pencil holds once it has factorised
 * nshift shifts in `precision` and, for ncv > 0, run an eigensolve with ncv basis
 * vectors: the plan's copies of A and B, the factors and the solve and Krylov
 * workspaces.  Computed from the sizes alone (nothing is allocated); the serving
 * queue below admits requests by it.
 */
int kore_plan_estimate_bytes(const kore_pencil_desc *desc, int precision, int nshift, int ncv, int64_t *bytes);

/*
 * Serving: a queue of eigen and forced solves of different pencils run by `workers`
 * host threads, each on its own plan and CUDA stream, admitted by device memory.
 * There is no counterpart in the reference, which runs one bin/solve.py process per
 * problem; a request does what one such run does (eigen: kore_eigs at its target;
 * forced: kore_solve at its shift) and writes the same results.
 *
 *  - Admission: a request starts when the estimate of its plan (kore_plan_estimate_bytes)
 *    fits in hbm_budget next to the plans in use and cached; idle cached plans are
 *    freed oldest first to make room.  Requests start in arrival order, except that one
 *    which does not fit yet does not hold back later ones that do (until it has waited
 *    longer than 200 ms, after which nothing new starts before it).
 *  - Continuous batching: eigen requests with the same non-zero pencil_key and
 *    precision run together in the factor slots of one plan (the engine of
 *    kore_eigs_shifts, four slots), sharing every launch; one that arrives while others
 *    of its pencil run takes the next free slot instead of starting a plan of its own.
 *  - Factor cache: requests with the same non-zero pencil_key share uploaded plans; a
 *    forced request whose (key, shift, precision) matches an idle cached plan skips the
 *    factorisation, and an eigen request reuses a slot that still holds its target's
 *    factors.  pencil_key = 0: the plan is freed after the request.
 *  - The caller keeps the pencil arrays, the right-hand side and the output buffers
 *    alive until kore_batch_poll reports the request finished.
 *  - A result does not depend on what else is running: each request runs on its own
 *    plan, and every kernel reduces in a fixed order.
 */
#define KORE_REQ_EIGEN  0
#define KORE_REQ_FORCED 1

typedef struct kore_batch kore_batch;

typedef struct {
    int32_t kind;                     /* KORE_REQ_EIGEN or KORE_REQ_FORCED */
    const kore_pencil_desc *pencil;   /* read when the request starts */
    uint64_t pencil_key;              /* caller's name for the pencil (0: no sharing) */
    int32_t precision;                /* KORE_PREC_* */
    double sigma_re, sigma_im;        /* forced: the shift; eigen: the target (opts.target_*) */
    kore_eps_opts opts;               /* eigen */
    const double *rhs;                /* forced: n complex right-hand side */
    double rhs_scale;                 /* forced: solves with rhs / rhs_scale (0 means 1) */
    double refine_tol;                /* forced, mixed precision (<= 0: 1e-14) */
    double *x;                        /* forced: n complex solution */
    double *evals;                    /* eigen: 2 * max_pairs doubles */
    double *evecs;                    /* eigen: NULL or 2 * n * max_pairs doubles */
    int32_t max_pairs;
    int32_t *nconv;                   /* eigen: converged pairs */
    double *timing_ms;                /* NULL or 3 doubles: queued, running, submit to finish */
    kore_stats *stats;                /* eigen: NULL or the solve's statistics */
} kore_request;

/* hbm_budget <= 0: 90% of the device's free memory at creation. */
int kore_batch_create(int device, int64_t hbm_budget, int workers, kore_batch **batch);
/* Copies *req (not the arrays it points to) and returns a ticket. */
int kore_batch_submit(kore_batch *batch, const kore_request *req, uint64_t *ticket);
/*
 * KORE_OK when the request has finished (*status = its status; the ticket is then
 * released), KORE_EPENDING when it has not after wait_ms milliseconds (-1: wait).
 */
int kore_batch_poll(kore_batch *batch, uint64_t ticket, int wait_ms, int *status);
/* out[9]: submitted, finished, running, queued, device bytes in plans, factor-cache
 * hits, plans created, plans freed to make room, eigen requests that joined a running
 * engine */
int kore_batch_stats(kore_batch *batch, int64_t *out);
/* Waits for running requests, cancels queued ones (KORE_ECANCELLED), frees all plans. */
int kore_batch_destroy(kore_batch *batch);

/*
 * Self-test of the tensor-core complex64 GEMM that the mixed-precision factorisation
 * uses (tcgen05, 3xTF32): nmat seeded S x S products, one and two per job, with and
 * without accumulation into C, checked against an FP64 product on the device.
 * *max_rel_err = max over entries of |C - C_fp64| / sum_k |a_ik| |b_kj|.
 * No counterpart in the reference; a diagnostic for the kernel.
 */
int kore_tc_selftest(int device, int S, int nmat, double *max_rel_err);

/*
 * Multiplication operator of the Gegenbauer (ultraspherical) basis, computed on
 * `device`: M multiplies a C^(lam) series by the function whose N C^(lam) coefficients
 * are a0 (lam >= 0; lam = 0 is the Chebyshev basis).  M is banded with half-width
 * h >= (index of the last nonzero of a0) + 1; band receives N (2h + 1) doubles,
 * band[(d + h) N + j] = M[j, j + d] for |d| <= h (0 outside the matrix).  Replaces Mlam
 * (bin/utils.py:962-1051), which bin/submatrices.py applies to every radial operator.
 */
int kore_gegenbauer_mult(int device, int N, const double *a0, double lam, int h, double *band);

/*
 * Flow diagnostics of velocity eigenvectors in a spherical shell (ricb in (0, 1),
 * rcmb = 1), computed on `device`: for nvec vectors x, each npol poloidal blocks (degrees
 * lpol) followed by ntor toroidal blocks (degrees ltor) of N complex Chebyshev
 * coefficients (the velocity part of a solution in bin/assemble.py's order), out
 * receives per vector and block the radial integrals of the kinetic energy, of
 * integral(u . lap u) and of the internal dissipation (3 doubles, blocks in the order
 * given).  Replaces flow_worker of bin/utils4pp.py:426-488, which bin/spin_doctor.py
 * runs over the degrees in a process pool; the sums over degrees, the scaling by
 * OmgTau Ek and the power-balance residuals are kore_gb300.diagnostics'.
 */
/*
 * Values and column indices of a block-structured pencil matrix assembled on the GPU
 * (bin/assemble.py:606-1176: A and B from the radial operators of bin/submatrices.py).
 * Unknowns in nrowblk blocks of n1.  ops: nops dense n1 x n1 complex radial operators,
 * row-major.  Block (R, C) of the matrix is sum_e coef_e op_e over the entries
 * e in [ent_ptr[R], ent_ptr[R+1]) with ent_col[e] = C (ent_op, ent_coef complex), except
 * that the first bc_g[R] rows of block R are its boundary rows, bc_vals + bc_ptr[R]
 * (bc_g[R] x n1 complex, row-major, in the columns of block R).  The sparsity pattern is
 * given per signature: row block R uses signature sig_of[R], whose local row i has the
 * entries sig_pat[sig_rowptr[s (n1+1) + i] .. sig_rowptr[s (n1+1) + i + 1]) as pairs
 * (block offset dC, local column j), column (R + dC) n1 + j, in increasing column order.
 * indptr (nrows + 1 = nrowblk n1 + 1, host) must hold the row lengths those patterns
 * give; indices (int32) and values (complex) receive the nnz entries (host arrays).
 * Synchronous; every array is checked against the others before the device is touched.
 */
int kore_assemble_blocks(int device, int n1, int nops, const double *ops, int64_t nrowblk,
                         const int32_t *sig_of, int nsig, const int32_t *sig_rowptr, int64_t npat,
                         const int32_t *sig_pat, const int64_t *ent_ptr, const int32_t *ent_col,
                         const int32_t *ent_op, const double *ent_coef, const int32_t *bc_g,
                         const int64_t *bc_ptr, int64_t bc_len, const double *bc_vals,
                         const int64_t *indptr, int64_t nnz, int32_t *indices, double *values);

int kore_flow_diagnostics(int device, int N, double ricb, int npol, const int32_t *lpol, int ntor,
                          const int32_t *ltor, const double *x, int nvec, double *out);

/* Number of kernels this library launched since load (for launch accounting). */
int64_t kore_kernel_launches(void);

const char *kore_status_string(int status);

int kore_plan_destroy(kore_plan *plan);

#ifdef __cplusplus
}
#endif
#endif /* KORE_GPU_H */
