// Internal plan structure and cross-file declarations of libkoregpu.
#pragma once

#include <vector>
#include "kore_common.cuh"

// Device-side state of the FP64 refinement loop and solve counters.
struct IrState {
    int done;          // current refinement finished
    int nan;           // a residual was NaN/Inf
    int iters;         // corrections applied (total)
    int iters_cur;     // corrections of the current application
    int iters_max;     // worst corrections of one application
    int applies;       // applications of the inverse
    int sweeps;        // sweeps that ran
    int pad_;
    double prev;       // previous eta of the current application
    double eta_max;    // worst final eta (an application that ran out of corrections: its last measured eta)
    int sweeps_total;  // sweeps that ran since the plan was created (kept by kore_ir_reset)
    int pad2_;
};

// One level of the block cyclic reduction.  Couplings of levels >= 1 are dense S x S
// blocks in kore_plan::d_LU: L of position q at lu_L + q, U at lu_U + q (block units).
struct BcrLevel {
    int Kl;          // active blocks
    int stride;      // original index of position q is q * stride
    int nodd;        // eliminated at this level: positions 1, 3, ...
    int neven;       // surviving: positions 0, 2, ...
    int64_t lu_L, lu_U;        // this level's couplings (-1 at level 0: they come from the CSR)
    int64_t lu_nL, lu_nU;      // next level's couplings (-1 when the next level is the top)
};

// Rows with more stored values (split A + B) than this are given a whole warp in the
// sparse products (the dense tau-method boundary rows); the others get one thread.
constexpr int kKoreLongRow = 128;

// The pencil is stored l-major and padded: block i (of nblocks K) occupies padded
// slots [i*S, (i+1)*S) where S is the largest block size rounded up to a multiple of 4;
// slots past the block's own size are identity rows/columns with zero right-hand side.
struct kore_plan {
    int device = 0;
    cudaStream_t stream = nullptr;
    int num_sms = 0;

    int64_t n = 0;        // unknowns (sizmat)
    int K = 0;            // blocks
    int S = 0;            // padded block size
    int64_t np = 0;       // K*S
    std::vector<int> bsz, boff;

    // A and B in l-major padded numbering (rows and columns)
    int *d_arow = nullptr, *d_acol = nullptr, *d_asplit = nullptr;
    double2 *d_aval = nullptr;
    int64_t a_nnz = 0;
    int *d_brow = nullptr, *d_bcol = nullptr;
    double *d_bval = nullptr;
    int64_t b_nnz = 0;
    bool has_b = false;
    int64_t *d_slot2orig = nullptr;   // np: original index or -1 for a pad slot
    // A for the sparse products, as a real matrix: row p holds the entries with a
    // nonzero real part (value Re a) in [srow[p], smid[p]) and those with a nonzero
    // imaginary part (value Im a) in [smid[p], srow[p+1]), so A x costs two real
    // multiply-adds per stored value (most entries of A are real or imaginary)
    int *d_srow = nullptr, *d_smid = nullptr, *d_scol = nullptr;
    double *d_sval = nullptr;
    int64_t s_nnz = 0;
    int *d_long_rows = nullptr;       // rows with more than kKoreLongRow stored values (A + B): a warp each
    int nlong = 0;
    int *d_bsz = nullptr;             // K

    // factorisation: block cyclic reduction (factor.cu).  Level l has lev[l].Kl active
    // blocks i = q * 2^l; the odd positions are eliminated, the even ones carry on.
    int prec = -1;
    bool factored = false;
    // factorised shifts: every factor buffer holds shift_cap sets, shift s at offset s * stride
    int nshift = 0, shift_cap = 0;
    // factor window: the shifts [fw_lo, fw_lo + fw_n) that the factorisation kernels work
    // on (all of them for kore_factor_shifts, one for a slot refill)
    int fw_lo = 0, fw_n = 0;
    int sweep_cps = 0;                // CTAs per SM of the last sweep (autotuned per plan shape)
    int sweep_chunk = 0;              // its ring chunk bytes
    std::vector<double2> sigmas;      // host copy of the shifts
    std::vector<double> minfs;        // ||A - sigma_s B||_inf per shift
    double2 *d_sigma = nullptr;       // device copy of the shifts
    double *d_minf = nullptr;
    double sigma_re = 0, sigma_im = 0;   // shift 0 (the eigensolver's target)
    double minf = 0;                     // ||A - sigma_0 B||_inf
    size_t factor_elt = 0;            // bytes of one complex element of the factors
    int nlev = 0;                     // reduction levels (the top block is solved after them)
    std::vector<struct BcrLevel> lev; // host copy of the level table
    struct BcrLevel *d_lev = nullptr; // device copy
    int64_t lu_mats = 0;              // dense coupling matrices of levels >= 1
    int nodd_max = 1;                 // largest number of blocks eliminated at one level
    // S x S column-major blocks, indexed by original block number, per shift
    void *d_Dinv = nullptr, *d_Gm = nullptr, *d_Hm = nullptr, *d_Dw = nullptr;
    void *d_LU = nullptr;             // lu_mats blocks per shift
    void *d_T = nullptr;              // nodd_max x (S x 2S) Gauss-Jordan work [D | I] per shift, column-major
    double *d_rscale = nullptr;       // np row equilibration factors per shift
    int *d_piv = nullptr;             // nodd_max x S per shift: pivot row chosen for column k
    int *d_pidx = nullptr;            // nodd_max x S per shift: position of a row in the current panel or -1
    int *d_used = nullptr;            // nodd_max x S per shift: row already used as a pivot
    // Level-0 couplings (the entries of a block's rows in the columns of its two
    // neighbours) as padded rows, tile by tile: entry k of row r of tile t of block i at
    // ((i * ntile + t) * ell_w + k) * 32 + r % 32, ntile = ceil(S / 32).  The first
    // reduction updates the even blocks' right-hand sides from them, and the last stage
    // of the back substitution forms the odd blocks' right-hand sides from them.
    int ell_w = 0;                    // padded width (multiple of 8) of a coupling row
    int64_t ell_rows = 0;             // K x ntile x 32
    int64_t ell_nnz = 0;              // coupling entries (without the padding)
    // Level-0 couplings of the odd blocks j (rows of block j, columns of block j-1 for
    // side 0 and of block j+1 for side 1) by column, for G_j = D_j^-1 L_j and
    // H_j = D_j^-1 U_j: column c of (odd index o, side) holds the entries
    // [cc_ptr[(2 o + side) (S + 1) + c], ... + c + 1) with row k in the block (cc_row)
    // and the entry of A in the permuted CSR (cc_src).
    int *d_cc_ptr = nullptr, *d_cc_row = nullptr, *d_cc_src = nullptr;
    int *d_ell_col = nullptr;         // padded slot of the coupled unknown, -1 for padding
    int *d_ell_src = nullptr;         // entry of A in the permuted CSR, -1 for padding
    void *d_ell_val = nullptr;        // per shift: rscale_row * A entry, factor precision
    // complex64 factorisation: TF32 split planes and job table of the tensor-core
    // even-block updates (gemm_tc.cu), sized for the largest level
    void *d_tcplanes = nullptr;
    void *d_tctab = nullptr;

    int64_t f_stride() const { return (int64_t)K * S * S; }
    int64_t lu_stride() const { return lu_mats * (int64_t)S * S; }
    int64_t t_stride() const { return (int64_t)nodd_max * 2 * S * S; }
    int64_t p_stride() const { return (int64_t)nodd_max * S; }
    int64_t ell_stride() const { return ell_rows * ell_w; }
    // stages of one sweep: A_l, B_l (l < nlev), the top block, C_l (nlev > l >= 1), E_0, C_0
    int sweep_stages() const { return nlev > 0 ? 3 * nlev + 2 : 1; }

    // solve workspace (padded, complex128 unless noted)
    double2 *d_v[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
    // per shift (shift_cap sets of np): sweep vectors in factor precision, and the
    // complex128 right-hand side, solution and residual of a batched solve
    void *d_zlo = nullptr, *d_xlo = nullptr, *d_flo = nullptr;
    double2 *d_bb = nullptr, *d_xb = nullptr, *d_rb = nullptr;
    double *d_bn = nullptr, *d_rn = nullptr;   // per-shift ||b||_inf and ||r||_inf
    double *d_red = nullptr;          // reduction scratch (8192 doubles)
    double *d_part = nullptr;         // per-CTA maxima of the residual kernel (2 per CTA, per shift)
    double *h_red = nullptr;          // pinned host mirror
    int *d_err = nullptr;
    unsigned *d_bar = nullptr;
    int *d_cnt = nullptr;             // sweep completion counters (shift_cap x sweep_stages() x K)
    IrState *d_ir = nullptr;          // one per shift

    // Krylov-Schur workspace (per target: basis and restart buffer of ncv + 1 columns)
    double2 *d_V = nullptr;           // np x ks_cap
    double2 *d_Vtmp = nullptr;        // np x ks_cap
    double2 *d_ksx = nullptr;         // np x targets: gathered input vectors of the sparse products
    int64_t ks_cap = 0;               // columns of d_V, d_Vtmp
    double2 *d_small = nullptr;       // projected problems, Gram-Schmidt coefficients and partial sums
    int ks_small_cap = 0;             // targets d_small holds
    // warm starts: per slot, the sum of the eigenvectors its last target returned (padded
    // order), kept across eigensolves of the plan
    double2 *d_warm = nullptr;        // np x warm_cap
    int warm_cap = 0;
    std::vector<char> warm_ok;        // slot s holds such a vector

    size_t bytes = 0;
    size_t factor_bytes = 0;          // bytes of the per-shift buffers
    int last_refine_iters = 0;
    double last_resid = 0;

    // kernel timing (kore_profile)
    bool prof = false;
    std::vector<cudaEvent_t> ev_pool;
    size_t ev_used = 0;
    std::vector<std::pair<int, size_t>> ev_marks;   // (kind, index of the start event)
    // kinds: 0 sweep, 1 factorisation, 2 sparse products (B x, residuals), 3 Krylov
    // orthogonalisation, 4 projected Schur problem and restart
    double prof_ms[5] = {0, 0, 0, 0, 0};
    long long prof_n[5] = {0, 0, 0, 0, 0};
    int sweeps_at_enable = 0;
};

// record a start (begin = true) or stop event of a timed region of `kind`
int kore_prof_mark(kore_plan *p, int kind, bool begin);
int kore_prof_collect(kore_plan *p);

// plan.cu
int kore_check_device_error(kore_plan *p);
int kore_alloc(kore_plan *p, void **ptr, size_t bytes);

// factor.cu
void kore_build_levels(kore_plan *p);
// factorise A - sigma_s B for nshift shifts (interleaved re, im) at once
int kore_factor_impl(kore_plan *p, int nshift, const double *sigmas, int precision);
// re-factorise shift `slot` of a factorised plan for a new shift, in the plan's
// precision; the other shifts' factors are kept
int kore_factor_slot(kore_plan *p, int slot, double sigma_re, double sigma_im);

// gemm_tc.cu: tensor-core (tcgen05, 3xTF32) even-block update of a level >= 1, complex64
int kore_even_update_tc(kore_plan *p, const BcrLevel &lv);
// G_j, H_j of the odd blocks with one refinement step (level0: G0, H0 already formed
// from the sparse couplings)
int kore_gh_update_tc(kore_plan *p, const BcrLevel &lv, int level0);
void kore_tc_level_bytes(const kore_plan *p, int cap, int64_t *plane_bytes, int64_t *table_bytes);

// sweep.cu
// x_s = (A - sigma_s B)^-1 b_s for every factorised shift s on padded l-major
// complex128 vectors (device; shift s at offset s * np), refined in FP64 when the
// factors are complex64 (asynchronous; counters in the plan's per-shift IrState).
// live_mask: only the shifts s < 32 whose bit is set are solved (the others' x is left
// as it is); shifts past 31 are always solved.
// shift_tols (host, nshift entries, may be null): per-shift refinement tolerances in
// place of tol (entries <= 0 use tol).
int kore_apply_inverse(kore_plan *p, const double2 *b, double2 *x, double tol, unsigned live_mask = ~0u,
                       const double *shift_tols = nullptr);
int kore_ir_reset(kore_plan *p);
int kore_ir_read(kore_plan *p, IrState *out);
// once per plan, before the sparse products run: their launch attributes
int kore_spmv_prepare(kore_plan *p);
// y = B x on padded vectors
int kore_spmv_b(kore_plan *p, const double2 *x, double2 *y);
// y_s = B x_s for the factorised shifts s in live_mask (vectors at offset s * np)
int kore_spmv_b_shifts(kore_plan *p, const double2 *x, double2 *y, unsigned live_mask);
// y_s = A x_s for the factorised shifts s in live_mask
int kore_spmv_a_shifts(kore_plan *p, const double2 *x, double2 *y, unsigned live_mask);
// y = A x - lam B x on padded vectors
int kore_spmv_pencil(kore_plan *p, double lre, double lim, const double2 *x, double2 *y);
int kore_gather(kore_plan *p, const double2 *orig, double2 *padded);
int kore_scatter(kore_plan *p, const double2 *padded, double2 *orig);
// nshift vectors at once (original order: shift s at s * n; padded: at s * np)
int kore_gather_shifts(kore_plan *p, const double2 *orig, double2 *padded);
int kore_scatter_shifts(kore_plan *p, const double2 *padded, double2 *orig);

// eigs.cu
// ntarget Krylov-Schur runs, targets 0 .. nshift-1 around the factorised shifts, the
// others admitted into slots as earlier ones finish
int kore_eigs_impl(kore_plan *p, int ntarget, const kore_eps_opts *o, double *evals, double *evecs,
                   int max_pairs, int *nconv, kore_stats *st);

// One target of the batched eigensolve engine: its options and where its results go.
struct EigsTarget {
    kore_eps_opts opts{};
    double *evals = nullptr;       // 2 * max_pairs doubles
    double *evecs = nullptr;       // NULL or 2 * n * max_pairs doubles
    int max_pairs = 0;
    int *nconv = nullptr;
    kore_stats *stats = nullptr;   // may be NULL
    void *tag = nullptr;           // the source's handle of the target
    int reused = 0;                // set by the engine: the slot already held this shift's factors
    int warm_started = 0;          // set by the engine: started from the slot's warm vector
};
// Supplier of targets to kore_eigs_engine (called from the engine's thread).
struct EigsSource {
    // a target for a free slot, or false when there is none now
    virtual bool next(EigsTarget *t) = 0;
    // the target's results are written; status KORE_OK, KORE_ENOCONV, KORE_ENAN or the
    // error that ended it
    virtual void finished(const EigsTarget &t, int status) = 0;
    virtual ~EigsSource() = default;
};
// Runs Krylov-Schur solves in the plan's nshift factor slots until every slot is idle
// and the source has nothing more.  Slot s holds a usable factorisation of shift
// sigmas[s] when valid[s] (may be null: none; on return, the slots' state); a target is
// placed in a free slot that holds its shift if there is one, else its shift is
// factorised in a free slot.  Slots hold bases of max_ncv + 1 vectors; a target with a
// larger ncv is handed back with KORE_EINVAL.
int kore_eigs_engine(kore_plan *p, EigsSource *src, bool *valid, int max_ncv);
// factor storage for nslot shifts in `precision`, none factorised yet: the slots of
// kore_eigs_engine
int kore_factor_reserve(kore_plan *p, int nslot, int precision);
