// Factorisation of A - sigma*B by block cyclic reduction over the l-major blocks.
//
// The row-equilibrated pencil R(A - sigma B) is block tridiagonal with diagonal
// blocks D_i and couplings L_i (to block i-1) and U_i (to block i+1).  One reduction
// level eliminates the blocks at odd positions j of the active sequence:
//
//     Gauss-Jordan on [D_j | L_j | U_j | I]  ->  [I | G_j | H_j | D_j^-1]
//          G_j = D_j^-1 L_j,   H_j = D_j^-1 U_j
//     for the even neighbours i (odd neighbours jl = left, jr = right):
//          D_i <- D_i - L_i H_jl - U_i G_jr
//          L_i <- -L_i G_jl        (couples i to the even block left of jl)
//          U_i <- -U_i H_jr        (couples i to the even block right of jr)
//
// which halves the number of active blocks; after ceil(log2 K) levels one block is
// left and only its inverse is formed.  All blocks of a level are independent, so
// every kernel below is batched over the blocks of the level: the work of one
// factorisation is a few hundred launches of GPU-wide batched dense kernels instead
// of a chain of K dependent block steps.  Level 0 takes D, L, U from the CSR
// (L and U sparse: the even-block update is a sparse x dense product); the dense
// updates of the higher levels are batched complex GEMMs.
//
// Gauss-Jordan is blocked: one CTA per block reduces a panel of NB columns in shared
// memory (pivot search over the rows not yet used as pivots, in-place elimination that
// turns the panel into the columns of the accumulated elementary transform E), then the
// trailing columns t of every block are updated by t <- E t, i.e.
// t[r] += sum_c E[r,c] t[piv_c], with the pivot rows themselves replaced.  Rows are
// never swapped: the pivot row of column k is recorded and the outputs are gathered
// by it.  Pivoting stays inside each diagonal block.
//
// Many shifts (forcing frequencies, targets) of one pencil are factorised together:
// every kernel carries the shift as one more grid dimension, and shift s uses its own
// row scales and factor set at offset s * stride.
//
// This replaces the sparse LU that SLEPc's ST sinvert / PETSc's PCLU build inside
// bin/solve.py:123 and :227; the ordering (odd-even elimination of l-blocks) is what
// exposes the parallelism.
#include "kore_internal.cuh"
#include <climits>
#include <algorithm>

namespace {

// Device view of the plan for the factorisation kernels; shift s uses offset
// s * (f|lu|t|p|rs)_stride into the per-shift buffers.
template <typename C>
struct FV {
    int S, K;
    int64_t np;
    const int *arow, *acol, *asplit, *brow, *bcol, *bsz;
    const double2 *aval;
    const double *bval;
    int has_b;
    const double2 *sigma;
    double *rscale;
    C *Dinv, *G, *H, *Dw, *LU, *T;
    int *piv, *pidx, *used, *err;
    const int *cc_ptr, *cc_row, *cc_src;
    const int *ell_col;      // level-0 coupling rows of every block (kore_plan::d_ell_*)
    const C *ell_val;
    int ell_w;
    int64_t ell_stride;
    int64_t f_stride, lu_stride, t_stride, p_stride;
};

// View of the plan's factor storage starting at the factor window's first shift (shift
// fw_lo + s of the plan is shift s of the view).
template <typename C>
FV<C> make_fv(kore_plan *p) {
    FV<C> v;
    const int64_t lo = p->fw_lo;
    v.S = p->S; v.K = p->K; v.np = p->np;
    v.arow = p->d_arow; v.acol = p->d_acol; v.asplit = p->d_asplit; v.brow = p->d_brow; v.bcol = p->d_bcol;
    v.bsz = p->d_bsz; v.aval = p->d_aval; v.bval = p->d_bval; v.has_b = p->has_b ? 1 : 0;
    v.sigma = p->d_sigma + lo; v.rscale = p->d_rscale + lo * p->np;
    v.Dinv = static_cast<C *>(p->d_Dinv) + lo * p->f_stride(); v.G = static_cast<C *>(p->d_Gm) + lo * p->f_stride();
    v.H = static_cast<C *>(p->d_Hm) + lo * p->f_stride(); v.Dw = static_cast<C *>(p->d_Dw) + lo * p->f_stride();
    v.LU = static_cast<C *>(p->d_LU) + lo * p->lu_stride(); v.T = static_cast<C *>(p->d_T) + lo * p->t_stride();
    v.piv = p->d_piv + lo * p->p_stride(); v.pidx = p->d_pidx + lo * p->p_stride();
    v.used = p->d_used + lo * p->p_stride(); v.err = p->d_err;
    v.cc_ptr = p->d_cc_ptr; v.cc_row = p->d_cc_row; v.cc_src = p->d_cc_src;
    v.ell_col = p->d_ell_col; v.ell_val = static_cast<const C *>(p->d_ell_val) + lo * p->ell_stride();
    v.ell_w = p->ell_w;
    v.ell_stride = p->ell_stride();
    v.f_stride = p->f_stride(); v.lu_stride = p->lu_stride(); v.t_stride = p->t_stride(); v.p_stride = p->p_stride();
    return v;
}

// Row equilibration by powers of two (exact): rscale[p] = 2^-e with
// e = exponent of max(max_e |a_pe|, |sigma| max_e |b_pe|); also the row 1-norms of
// |A| + |sigma||B| whose maximum bounds ||A - sigma B||_inf.  Shift = blockIdx.y;
// per-CTA maxima to red[s * gridDim.x + blockIdx.x].
template <typename C>
__global__ void k_rowinfo(FV<C> v, double *__restrict__ red) {
    const int s = blockIdx.y;
    const double2 sg = v.sigma[s];
    const double sabs = sqrt(abs2(sg));
    double *rscale = v.rscale + (int64_t)s * v.np;
    double mx = 0.0;
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < v.np; p += (int64_t)gridDim.x * blockDim.x) {
        double am = 0.0, sum = 0.0;
        for (int e = v.arow[p]; e < v.arow[p + 1]; ++e) {
            const double t = sqrt(abs2(v.aval[e]));
            am = fmax(am, t);
            sum += t;
        }
        if (v.has_b)
            for (int e = v.brow[p]; e < v.brow[p + 1]; ++e) {
                const double t = sabs * fabs(v.bval[e]);
                am = fmax(am, t);
                sum += t;
            }
        rscale[p] = (am > 0.0) ? ldexp(1.0, -ilogb(am)) : 1.0;
        mx = fmax(mx, sum);
    }
    mx = warp_max_d(mx);
    __shared__ double sm[32];
    if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = mx;
    __syncthreads();
    if (threadIdx.x < 32) {
        double t = (threadIdx.x < (blockDim.x >> 5)) ? sm[threadIdx.x] : 0.0;
        t = warp_max_d(t);
        if (threadIdx.x == 0) red[(int64_t)s * gridDim.x + blockIdx.x] = t;
    }
}

// Values of the padded level-0 coupling rows for every shift: rscale_row * A entry in
// the factor precision (grid (x, shift)).
template <typename C>
__global__ void k_ell_fill(int64_t ell_stride, int ell_w, int ntile, int S, int64_t np,
                           const int *__restrict__ src, const double2 *__restrict__ aval,
                           const double *__restrict__ rscale, C *__restrict__ val) {
    const int64_t s = blockIdx.y;
    for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < ell_stride;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const int e = src[idx];
        C v = czero<C>();
        if (e >= 0) {
            const int64_t lane = idx & 31, tile = idx / 32 / ell_w;   // tile = block * ntile + t
            const int64_t bi = tile / ntile, t = tile - bi * ntile;
            const int64_t row = bi * S + t * 32 + lane;
            v = from_c128<C>(rscale[s * np + row] * aval[e]);
        }
        val[s * ell_stride + idx] = v;
    }
}

// Dw <- 0 with the identity on the padded diagonal of every block, all shifts.
template <typename C>
__global__ void k_Dw_init(FV<C> v, int nshift) {
    const int64_t SS = (int64_t)v.S * v.S, per = (int64_t)v.K * SS, total = per * nshift;
    for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const int64_t w = idx % per;
        const int64_t i = w / SS;
        const int64_t e = w - i * SS;
        const int c = (int)(e / v.S), r = (int)(e - (int64_t)c * v.S);
        v.Dw[idx] = (r == c && r >= v.bsz[i]) ? cone<C>() : czero<C>();
    }
}

// One warp per (shift, row): Dw_i[r, :] = rs_r (D_i - sigma B_i)[r, :] from the CSR.
// A and B entries of the same column are combined in FP64 and rounded once.
template <typename C>
__global__ void k_Dw_scatter(FV<C> v, int nshift) {
    const int lane = threadIdx.x & 31;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const int S = v.S;
    for (int64_t w = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5; w < v.np * nshift; w += nw) {
        const int64_t s = w / v.np, p = w - s * v.np;
        const int64_t i = p / S;
        const int r = (int)(p - i * S);
        const double2 sigma = v.sigma[s];
        const double rs = v.rscale[s * v.np + p];
        C *D = v.Dw + s * v.f_stride + i * (int64_t)S * S;
        const int eD = v.asplit[2 * p], eU = v.asplit[2 * p + 1];
        for (int e = eD + lane; e < eU; e += 32) D[r + (int64_t)(v.acol[e] - i * S) * S] = from_c128<C>(rs * v.aval[e]);
        __syncwarp();
        if (v.has_b)
            for (int e = v.brow[p] + lane; e < v.brow[p + 1]; e += 32) {
                const int c = v.bcol[e];
                int lo = eD, hi = eU;   // matching A entry: binary search in the sorted D segment
                while (lo < hi) {
                    const int mid = (lo + hi) >> 1;
                    if (v.acol[mid] < c) lo = mid + 1; else hi = mid;
                }
                const double2 a = (lo < eU && v.acol[lo] == c) ? v.aval[lo] : mk(0.0, 0.0);
                D[r + (int64_t)(c - i * S) * S] = from_c128<C>(rs * (a - v.bval[e] * sigma));
            }
    }
}

// T_o = [Dw_j | I] for the odd blocks j of level lv, all shifts.  stride 0 selects
// block 0 (the top of the reduction).
template <typename C>
__global__ void k_T_fill(FV<C> v, BcrLevel lv, int nodd, int nshift) {
    const int S = v.S;
    const int64_t SS = (int64_t)S * S, per = 2 * SS, pershift = (int64_t)nodd * per, total = pershift * nshift;
    for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const int64_t s = idx / pershift;
        const int64_t ws = idx - s * pershift;
        const int64_t o = ws / per;
        const int64_t e = ws - o * per;
        const int part = (int)(e / SS);
        const int64_t w = e - (int64_t)part * SS;
        const int64_t q = 2 * o + 1;               // position of the odd block
        const int64_t j = q * lv.stride;           // original block
        C val;
        if (part == 0) val = v.Dw[s * v.f_stride + j * SS + w];
        else {
            const int c = (int)(w / S), r = (int)(w - (int64_t)c * S);
            val = (r == c) ? cone<C>() : czero<C>();
        }
        v.T[s * v.t_stride + o * per + e] = val;
    }
}

// Panel reduction of columns [k0, k0+nb) of T_o; one CTA per (odd block o = blockIdx.x,
// shift = blockIdx.y).
template <typename C, int NB>
__global__ void __launch_bounds__(1024) k_panel(FV<C> v, int k0) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int S = v.S;
    C *P = reinterpret_cast<C *>(smem_raw);
    int *u = reinterpret_cast<int *>(P + (size_t)S * NB);
    __shared__ C prow[NB];
    __shared__ double rv[32];
    __shared__ int ri[32];
    __shared__ int s_p;
    __shared__ C s_dinv;
    __shared__ int s_piv[NB];
    const int64_t o = blockIdx.x, sh = blockIdx.y;
    C *T = v.T + sh * v.t_stride + o * 2 * (int64_t)S * S;
    int *piv = v.piv + sh * v.p_stride + o * S, *pidx = v.pidx + sh * v.p_stride + o * S;
    int *used = v.used + sh * v.p_stride + o * S;
    const int tid = threadIdx.x, nt = blockDim.x;
    const int nb = min(NB, S - k0);

    for (int idx = tid; idx < S * nb; idx += nt) P[idx] = T[(int64_t)k0 * S + idx];
    for (int r = tid; r < S; r += nt) u[r] = (k0 == 0) ? 0 : used[r];
    __syncthreads();

    int c = 0;
    for (; c < nb; ++c) {
        double best = -1.0;
        int bi = INT_MAX;
        for (int r = tid; r < S; r += nt)
            if (!u[r]) {
                const double val = (double)abs2(P[c * S + r]);
                if (val > best) { best = val; bi = r; }
            }
        for (int off = 16; off > 0; off >>= 1) {
            const double ov = __shfl_down_sync(0xffffffffu, best, off);
            const int oi = __shfl_down_sync(0xffffffffu, bi, off);
            if (ov > best || (ov == best && oi < bi)) { best = ov; bi = oi; }
        }
        if ((tid & 31) == 0) { rv[tid >> 5] = best; ri[tid >> 5] = bi; }
        __syncthreads();
        if (tid < 32) {
            const int nw = nt >> 5;
            best = (tid < nw) ? rv[tid] : -1.0;
            bi = (tid < nw) ? ri[tid] : INT_MAX;
            for (int off = 16; off > 0; off >>= 1) {
                const double ov = __shfl_down_sync(0xffffffffu, best, off);
                const int oi = __shfl_down_sync(0xffffffffu, bi, off);
                if (ov > best || (ov == best && oi < bi)) { best = ov; bi = oi; }
            }
            if (tid == 0) {
                int p = bi;
                if (p >= S || !(best > 0.0)) {
                    atomicCAS(v.err, 0, KORE_DEVERR_PIVOT);
                    p = -1;
                } else {
                    u[p] = 1;
                    s_dinv = cdiv(cone<C>(), P[c * S + p]);
                }
                s_p = p;
                s_piv[c] = p;
            }
        }
        __syncthreads();
        const int p = s_p;
        if (p < 0) break;
        const C dinv = s_dinv;
        if (tid < nb) prow[tid] = (tid == c) ? dinv : P[tid * S + p] * dinv;
        __syncthreads();
        for (int r = tid; r < S; r += nt) {
            const C mult = P[c * S + r];
            if (r == p) {
                for (int cc = 0; cc < nb; ++cc) if (cc != c) P[cc * S + r] = prow[cc];
            } else {
                for (int cc = 0; cc < nb; ++cc) if (cc != c) P[cc * S + r] = cfms(P[cc * S + r], mult, prow[cc]);
            }
            P[c * S + r] = (r == p) ? dinv : -(mult * dinv);
        }
        __syncthreads();
    }
    const int done = c;
    for (int idx = tid; idx < S * nb; idx += nt) T[(int64_t)k0 * S + idx] = P[idx];
    for (int r = tid; r < S; r += nt) { used[r] = u[r]; pidx[r] = -1; }
    __syncthreads();
    if (tid < done) { piv[k0 + tid] = s_piv[tid]; pidx[s_piv[tid]] = tid; }
    // after a zero pivot the remaining columns keep an in-range row index so that the
    // update and extraction kernels stay in bounds (the error flag is already set)
    if (tid >= done && tid < nb) piv[k0 + tid] = 0;
}

// Trailing update of TW columns per CTA (blockIdx.x) of odd block blockIdx.y, shift blockIdx.z.
template <typename C, int NB, int TW>
__global__ void __launch_bounds__(256) k_update(FV<C> v, int k0, int nb, int col_begin, int col_end) {
    __shared__ C tp[TW][NB];
    const int S = v.S;
    const int64_t o = blockIdx.y, sh = blockIdx.z;
    C *T = v.T + sh * v.t_stride + o * 2 * (int64_t)S * S;
    const int *piv = v.piv + sh * v.p_stride + o * S, *pidx = v.pidx + sh * v.p_stride + o * S;
    const int j0 = col_begin + blockIdx.x * TW;
    const int tw = min(TW, col_end - j0);
    for (int idx = threadIdx.x; idx < TW * NB; idx += blockDim.x) {
        const int t = idx / NB, c = idx - t * NB;
        tp[t][c] = (t < tw && c < nb) ? T[piv[k0 + c] + (int64_t)(j0 + t) * S] : czero<C>();
    }
    __syncthreads();
    const C *E = T + (int64_t)k0 * S;
    for (int r = threadIdx.x; r < S; r += blockDim.x) {
        C er[NB];
#pragma unroll
        for (int c = 0; c < NB; ++c) er[c] = (c < nb) ? E[r + (int64_t)c * S] : czero<C>();
        const bool isp = pidx[r] >= 0;
        for (int t = 0; t < tw; ++t) {
            const int64_t idx = r + (int64_t)(j0 + t) * S;
            C acc = isp ? czero<C>() : T[idx];
#pragma unroll
            for (int c = 0; c < NB; ++c) acc = cfma(acc, er[c], tp[t][c]);
            T[idx] = acc;
        }
    }
}

// Solution rows by pivot: Dinv_j[k,:] = T[piv[k], S:2S)  (column-major S x S), all shifts.
template <typename C>
__global__ void k_extract(FV<C> v, BcrLevel lv, int nodd, int top, int nshift) {
    const int S = v.S;
    const int64_t SS = (int64_t)S * S, pershift = (int64_t)nodd * SS, total = pershift * nshift;
    for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const int64_t sh = idx / pershift;
        const int64_t ws = idx - sh * pershift;
        const int64_t o = ws / SS;
        const int64_t w = ws - o * SS;
        const int c = (int)(w / S), k = (int)(w - (int64_t)c * S);
        const C *T = v.T + sh * v.t_stride + o * 2 * SS;
        const int p = v.piv[sh * v.p_stride + o * S + k];
        const int64_t j = top ? 0 : (2 * o + 1) * lv.stride;
        v.Dinv[sh * v.f_stride + j * SS + w] = T[p + (int64_t)(S + c) * S];
    }
}

// Level 0 update of the even blocks with their sparse couplings:
//   Dw_i -= rs (L_i H_jl + U_i G_jr),  L'_i = -rs L_i G_jl,  U'_i = -rs U_i H_jr.
// CTA = (chunk of kEvenCW columns, even index e, shift); one thread per row, which reads
// its row's coupling entries once, as padded rows (the level-0 rows of the sweep, with
// the row scale folded in), and accumulates the kEvenCW columns in registers.
constexpr int kEvenCW = 8;
template <typename C>
__global__ void __launch_bounds__(512) k_even_l0(FV<C> v, BcrLevel lv) {
    const int S = v.S;
    const int64_t SS = (int64_t)S * S;
    const int64_t e = blockIdx.y, sh = blockIdx.z;
    const int64_t q = 2 * e;                 // position = original block at level 0
    const bool outl = (lv.lu_nL >= 0) && q >= 2, outr = (lv.lu_nU >= 0) && q + 2 < lv.Kl;
    const int c0 = blockIdx.x * kEvenCW;
    const int cn = min(kEvenCW, S - c0);
    const int ntile = (S + 31) / 32;
    C *Di = v.Dw + sh * v.f_stride + q * SS;
    const C *G = v.G + sh * v.f_stride, *H = v.H + sh * v.f_stride;
    const C *Hl = H + (q - 1) * SS, *Gl = G + (q - 1) * SS, *Gr = G + (q + 1) * SS, *Hr = H + (q + 1) * SS;
    C *LU = v.LU + sh * v.lu_stride;
    const C *ev = v.ell_val + sh * v.ell_stride;
    for (int r = threadIdx.x; r < S; r += blockDim.x) {
        C dsum[kEvenCW], lsum[kEvenCW], usum[kEvenCW];
#pragma unroll
        for (int t = 0; t < kEvenCW; ++t) dsum[t] = lsum[t] = usum[t] = czero<C>();
        const int64_t ebase = ((q * ntile + r / 32) * (int64_t)v.ell_w) * 32 + (r & 31);
        for (int k = 0; k < v.ell_w; ++k) {
            const int col = v.ell_col[ebase + (int64_t)k * 32];
            if (col < 0) continue;
            const C a = ev[ebase + (int64_t)k * 32];
            const int64_t blk = col / S, cr = col - blk * S;
            if (blk < q) {   // left neighbour j = q - 1
#pragma unroll
                for (int t = 0; t < kEvenCW; ++t)
                    if (t < cn) {
                        const int64_t o = cr + (int64_t)(c0 + t) * S;
                        dsum[t] = cfma(dsum[t], a, Hl[o]);
                        if (outl) lsum[t] = cfma(lsum[t], a, Gl[o]);
                    }
            } else {         // right neighbour j = q + 1
#pragma unroll
                for (int t = 0; t < kEvenCW; ++t)
                    if (t < cn) {
                        const int64_t o = cr + (int64_t)(c0 + t) * S;
                        dsum[t] = cfma(dsum[t], a, Gr[o]);
                        if (outr) usum[t] = cfma(usum[t], a, Hr[o]);
                    }
            }
        }
#pragma unroll
        for (int t = 0; t < kEvenCW; ++t)
            if (t < cn) {
                const int64_t col = (int64_t)(c0 + t) * S;
                Di[r + col] = Di[r + col] - dsum[t];
                if (outl) LU[(lv.lu_nL + e) * SS + r + col] = -lsum[t];
                if (outr) LU[(lv.lu_nU + e) * SS + r + col] = -usum[t];
            }
    }
}

// One 64 x 64 tile (blockIdx.x, blockIdx.y) of Cm = [Cm] +- (A1 B1 + A2 B2) for
// column-major S x S complex operands (A2 may be null), 4 x 4 outputs per thread,
// FP64/FP32 CUDA cores.
constexpr int kGT = 64, kGK = 16;
template <typename C>
__device__ __forceinline__ void gemm_tile(const C *A1, const C *B1, const C *A2, const C *B2, C *Cm, int S,
                                          bool accumulate, bool negate) {
    __shared__ C As[kGK][kGT + 1];
    __shared__ C Bs[kGK][kGT + 1];
    const int m0 = blockIdx.x * kGT, n0 = blockIdx.y * kGT;
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;   // 16 x 16 threads
    C acc[4][4];
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) acc[a][b] = czero<C>();
    for (int pass = 0; pass < 2; ++pass) {
        const C *A = pass ? A2 : A1;
        const C *B = pass ? B2 : B1;
        if (!A) continue;
        for (int k0 = 0; k0 < S; k0 += kGK) {
            for (int idx = threadIdx.x; idx < kGK * kGT; idx += blockDim.x) {
                const int kk = idx / kGT, mm = idx - kk * kGT;
                const int gm = m0 + mm, gk = k0 + kk;
                As[kk][mm] = (gm < S && gk < S) ? A[gm + (int64_t)gk * S] : czero<C>();
                const int nn = idx / kGK, kb = idx - nn * kGK;
                const int gn = n0 + nn, gk2 = k0 + kb;
                Bs[kb][nn] = (gn < S && gk2 < S) ? B[gk2 + (int64_t)gn * S] : czero<C>();
            }
            __syncthreads();
#pragma unroll
            for (int kk = 0; kk < kGK; ++kk) {
                C av[4], bv[4];
#pragma unroll
                for (int a = 0; a < 4; ++a) av[a] = As[kk][tx + 16 * a];
#pragma unroll
                for (int b = 0; b < 4; ++b) bv[b] = Bs[kk][ty + 16 * b];
#pragma unroll
                for (int a = 0; a < 4; ++a)
#pragma unroll
                    for (int b = 0; b < 4; ++b) acc[a][b] = cfma(acc[a][b], av[a], bv[b]);
            }
            __syncthreads();
        }
    }
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) {
            const int gm = m0 + tx + 16 * a, gn = n0 + ty + 16 * b;
            if (gm < S && gn < S) {
                const int64_t idx = gm + (int64_t)gn * S;
                const C d = negate ? -acc[a][b] : acc[a][b];
                Cm[idx] = accumulate ? Cm[idx] + d : d;
            }
        }
}

// Batched dense update of the even blocks at levels >= 1 (complex128; the complex64
// factorisation runs it on the tensor cores, gemm_tc.cu), one GEMM job per
// (shift, even block, kind): kind 0: Dw_i -= L_q H_jl + U_q G_jr;  kind 1: L' = -L_q G_jl;
// kind 2: U' = -U_q H_jr.
template <typename C>
__global__ void __launch_bounds__(256) k_even_gemm(FV<C> v, BcrLevel lv, int job0) {
    const int S = v.S;
    const int64_t SS = (int64_t)S * S;
    const int job = job0 + blockIdx.z;
    const int per = 3 * lv.neven;
    const int64_t sh = job / per;
    const int jj = job - (int)sh * per;
    const int64_t e = jj / 3;
    const int kind = jj - 3 * (int)e;
    const int64_t q = 2 * e;
    const bool hasl = q >= 1, hasr = q + 1 < lv.Kl;
    const C *A1 = nullptr, *B1 = nullptr, *A2 = nullptr, *B2 = nullptr;
    C *Cm = nullptr;
    bool accumulate = false;
    C *LU = v.LU + sh * v.lu_stride;
    const C *G = v.G + sh * v.f_stride, *H = v.H + sh * v.f_stride;
    const C *Lq = LU + (lv.lu_L + q) * SS, *Uq = LU + (lv.lu_U + q) * SS;
    const int64_t jl = (q - 1) * lv.stride, jr = (q + 1) * lv.stride;
    if (kind == 0) {
        Cm = v.Dw + sh * v.f_stride + q * lv.stride * SS;
        accumulate = true;
        if (hasl) { A1 = Lq; B1 = H + jl * SS; }
        if (hasr) { A2 = Uq; B2 = G + jr * SS; }
    } else if (kind == 1) {
        if (lv.lu_nL < 0 || q < 2) return;
        Cm = LU + (lv.lu_nL + e) * SS;
        A1 = Lq; B1 = G + jl * SS;
    } else {
        if (lv.lu_nU < 0 || q + 2 >= lv.Kl) return;
        Cm = LU + (lv.lu_nU + e) * SS;
        A1 = Uq; B1 = H + jr * SS;
    }
    if (!A1) { A1 = A2; B1 = B2; A2 = nullptr; B2 = nullptr; }
    if (!A1) return;
    gemm_tile<C>(A1, B1, A2, B2, Cm, S, accumulate, true);
}

// G_j = D_j^-1 L_q and H_j = D_j^-1 U_q of the odd blocks of a level >= 1 (complex128;
// complex64 on the tensor cores), one job per (shift, odd block, G or H).
template <typename C>
__global__ void __launch_bounds__(256) k_gh_gemm(FV<C> v, BcrLevel lv, int job0) {
    const int S = v.S;
    const int64_t SS = (int64_t)S * S;
    const int job = job0 + blockIdx.z;
    const int64_t sh = job / (2 * lv.nodd);
    const int jj = job - (int)sh * 2 * lv.nodd;
    const int64_t o = jj / 2;
    const int which = jj - 2 * (int)o;
    const int64_t q = 2 * o + 1, j = q * lv.stride;
    if (which == 1 && q + 1 >= lv.Kl) return;   // no right neighbour: H_j is never read
    const C *Di = v.Dinv + sh * v.f_stride + j * SS;
    const C *Bm = v.LU + sh * v.lu_stride + ((which ? lv.lu_U : lv.lu_L) + q) * SS;
    C *Cm = (which ? v.H : v.G) + sh * v.f_stride + j * SS;
    gemm_tile<C>(Di, Bm, nullptr, nullptr, Cm, S, false, false);
}

// Level 0: G_j = D_j^-1 (R L_j) and H_j = D_j^-1 (R U_j) from the couplings by column:
// column c of G_j = sum over the entries (k, e) of column c of L_j of rs_k a_e D_j^-1[:, k]
// (D_j^-1 is the inverse of the row-scaled block, so this is D^-1 L of the unscaled
// system).  CTA = (chunk of kGhCW columns, odd index o, shift): the entries of one column
// are staged in shared memory, then one thread per row accumulates.
constexpr int kGhCW = 8;
constexpr int kGhBuf = 512;
template <typename C>
__global__ void __launch_bounds__(512) k_gh_l0(FV<C> v) {
    __shared__ int sk[kGhBuf];
    __shared__ C sv[kGhBuf];
    const int S = v.S;
    const int64_t SS = (int64_t)S * S;
    const int64_t o = blockIdx.y, sh = blockIdx.z, j = 2 * o + 1;
    const int c0 = blockIdx.x * kGhCW, c1 = min(S, c0 + kGhCW);
    const C *Di = v.Dinv + sh * v.f_stride + j * SS;
    const double *rs = v.rscale + sh * v.np + j * S;
    for (int side = 0; side < 2; ++side) {
        const int *ptr = v.cc_ptr + (2 * o + side) * (int64_t)(S + 1);
        C *out = (side ? v.H : v.G) + sh * v.f_stride + j * SS;
        for (int c = c0; c < c1; ++c) {
            C acc[4] = {czero<C>(), czero<C>(), czero<C>(), czero<C>()};   // rows r, r + nt, ...
            for (int b0 = ptr[c]; b0 < ptr[c + 1]; b0 += kGhBuf) {
                const int nb = min(kGhBuf, ptr[c + 1] - b0);
                __syncthreads();
                for (int t = threadIdx.x; t < nb; t += blockDim.x) {
                    const int k = v.cc_row[b0 + t];
                    sk[t] = k;
                    sv[t] = from_c128<C>(rs[k] * v.aval[v.cc_src[b0 + t]]);
                }
                __syncthreads();
#pragma unroll
                for (int h = 0; h < 4; ++h) {
                    const int r = threadIdx.x + h * blockDim.x;
                    if (r < S)
                        for (int t = 0; t < nb; ++t) acc[h] = cfma(acc[h], Di[r + (int64_t)sk[t] * S], sv[t]);
                }
            }
#pragma unroll
            for (int h = 0; h < 4; ++h) {
                const int r = threadIdx.x + h * blockDim.x;
                if (r < S) out[r + (int64_t)c * S] = acc[h];
            }
        }
    }
}

constexpr int kUpdTW = 8;

unsigned grid_for(int64_t work, int threads, int num_sms) {
    return (unsigned)std::max<int64_t>(1, std::min<int64_t>((work + threads - 1) / threads, 16LL * num_sms));
}

// Gauss-Jordan of the nodd work matrices T_o of every shift (all panels), then extraction.
template <typename C, int NB>
int gauss_jordan(kore_plan *p, const FV<C> &v, const BcrLevel &lv, int nodd, int top, int nshift) {
    const int S = p->S;
    const size_t smem = (size_t)S * NB * sizeof(C) + (size_t)S * sizeof(int);
    KORE_TRY(kore_allow_max_dyn_smem(k_panel<C, NB>, p->device));
    const int pthreads = std::min(1024, ((S + 31) / 32) * 32);
    for (int k0 = 0; k0 < S; k0 += NB) {
        const int nb = std::min(NB, S - k0);
        k_panel<C, NB><<<dim3(nodd, nshift), pthreads, smem, p->stream>>>(v, k0);
        KORE_LAUNCHED(1);
        const int cb = k0 + nb;
        // trailing columns: the rest of D, then the identity columns
        dim3 g(kore_div_up(2 * S - cb, kUpdTW), nodd, nshift);
        k_update<C, NB, kUpdTW><<<g, 256, 0, p->stream>>>(v, k0, nb, cb, 2 * S);
        KORE_LAUNCHED(1);
    }
    k_extract<C><<<grid_for((int64_t)nodd * S * S * nshift, 256, p->num_sms), 256, 0, p->stream>>>(v, lv, nodd, top,
                                                                                                nshift);
    KORE_LAUNCHED(1);
    KORE_CUDA_TRY(cudaGetLastError());
    return KORE_OK;
}

template <typename C, int NB>
int factor_levels(kore_plan *p) {
    const int S = p->S, K = p->K, ns = p->fw_n;
    const int64_t SS = (int64_t)S * S;
    cudaStream_t st = p->stream;
    const FV<C> v = make_fv<C>(p);
    // working diagonal blocks from the CSR
    k_Dw_init<C><<<grid_for((int64_t)K * SS * ns, 256, p->num_sms), 256, 0, st>>>(v, ns);
    k_Dw_scatter<C><<<grid_for(p->np * 32 * ns, 256, p->num_sms), 256, 0, st>>>(v, ns);
    KORE_LAUNCHED(2);
    for (int l = 0; l < p->nlev; ++l) {
        const BcrLevel &lv = p->lev[l];
        k_T_fill<C><<<grid_for((int64_t)lv.nodd * 2 * SS * ns, 256, p->num_sms), 256, 0, st>>>(v, lv, lv.nodd, ns);
        KORE_LAUNCHED(1);
        // D_j^-1 of the odd blocks by Gauss-Jordan on [D_j | I]
        KORE_TRY((gauss_jordan<C, NB>(p, v, lv, lv.nodd, 0, ns)));
        const int th = std::min(512, ((S + 31) / 32) * 32);   // rows per pass (S <= 1024: two passes at most)
        if (l == 0) {
            // G_j, H_j from the sparse couplings (complex64: refined on the tensor cores),
            // then the even blocks
            k_gh_l0<C><<<dim3(kore_div_up(S, kGhCW), lv.nodd, ns), th, 0, st>>>(v);
            KORE_LAUNCHED(1);
            if (sizeof(C) == sizeof(float2)) KORE_TRY(kore_gh_update_tc(p, lv, 1));
            dim3 g(kore_div_up(S, kEvenCW), lv.neven, ns);
            k_even_l0<C><<<g, th, 0, st>>>(v, lv);
            KORE_LAUNCHED(1);
        } else if (sizeof(C) == sizeof(float2)) {
            // complex64: tensor cores (3xTF32)
            KORE_TRY(kore_gh_update_tc(p, lv, 0));
            KORE_TRY(kore_even_update_tc(p, lv));
        } else {
            // complex128: FP64 CUDA cores
            const dim3 tg(kore_div_up(S, kGT), kore_div_up(S, kGT));
            const int gjobs = 2 * lv.nodd * ns;
            for (int j0 = 0; j0 < gjobs; j0 += 65535) {
                k_gh_gemm<C><<<dim3(tg.x, tg.y, std::min(65535, gjobs - j0)), 256, 0, st>>>(v, lv, j0);
                KORE_LAUNCHED(1);
            }
            const int jobs = 3 * lv.neven * ns;
            for (int j0 = 0; j0 < jobs; j0 += 65535) {
                k_even_gemm<C><<<dim3(tg.x, tg.y, std::min(65535, jobs - j0)), 256, 0, st>>>(v, lv, j0);
                KORE_LAUNCHED(1);
            }
        }
        KORE_CUDA_TRY(cudaGetLastError());
    }
    // the last active block (block 0): T = [Dw_0 | I]; stride 0 maps odd index 0 to block 0
    BcrLevel top{};
    top.Kl = 1;
    top.stride = 0;
    top.lu_L = top.lu_U = top.lu_nL = top.lu_nU = -1;
    k_T_fill<C><<<grid_for(2 * SS * ns, 256, p->num_sms), 256, 0, st>>>(v, top, 1, ns);
    KORE_LAUNCHED(1);
    KORE_TRY((gauss_jordan<C, NB>(p, v, top, 1, 1, ns)));
    return KORE_OK;
}

template <typename C>
int factor_dispatch(kore_plan *p) {
    const size_t cap = 220 * 1024;
    auto fits = [&](int nb) { return (size_t)p->S * nb * sizeof(C) + (size_t)p->S * sizeof(int) <= cap; };
    if (sizeof(C) == 8 && fits(32)) return factor_levels<C, 32>(p);
    if (fits(16)) return factor_levels<C, 16>(p);
    if (fits(8)) return factor_levels<C, 8>(p);
    if (fits(4)) return factor_levels<C, 4>(p);
    return KORE_EINVAL;
}

}  // namespace

// Level table of the reduction for K blocks.
void kore_build_levels(kore_plan *p) {
    p->lev.clear();
    std::vector<int> Ks;
    for (int Kl = p->K; Kl > 1; Kl = Kl - Kl / 2) Ks.push_back(Kl);
    p->nlev = (int)Ks.size();
    p->nodd_max = 1;
    int64_t lu = 0;
    std::vector<int64_t> offL(p->nlev + 1, -1), offU(p->nlev + 1, -1);
    for (int l = 1; l < p->nlev; ++l) {
        offL[l] = lu;
        lu += Ks[l];
        offU[l] = lu;
        lu += Ks[l];
    }
    int stride = 1;
    for (int l = 0; l < p->nlev; ++l) {
        BcrLevel lv;
        lv.Kl = Ks[l];
        lv.stride = stride;
        lv.nodd = Ks[l] / 2;
        lv.neven = Ks[l] - lv.nodd;
        lv.lu_L = offL[l];
        lv.lu_U = offU[l];
        lv.lu_nL = (l + 1 < p->nlev) ? offL[l + 1] : -1;
        lv.lu_nU = (l + 1 < p->nlev) ? offU[l + 1] : -1;
        p->lev.push_back(lv);
        p->nodd_max = std::max(p->nodd_max, lv.nodd);
        stride *= 2;
    }
    p->lu_mats = std::max<int64_t>(lu, 1);
}

namespace {

// (Re)allocate the per-shift buffers for `cap` shifts of elements of `elt` bytes.
int ensure_factor_storage(kore_plan *p, int cap, size_t elt) {
    if (p->factor_elt == elt && p->shift_cap >= cap) return KORE_OK;
    void **bufs[] = {&p->d_Dinv, &p->d_Gm, &p->d_Hm, &p->d_Dw, &p->d_LU, &p->d_T, &p->d_zlo, &p->d_xlo, &p->d_flo,
                     (void **)&p->d_rscale, (void **)&p->d_piv, (void **)&p->d_pidx, (void **)&p->d_used,
                     (void **)&p->d_sigma, (void **)&p->d_minf, (void **)&p->d_bb, (void **)&p->d_xb, (void **)&p->d_rb,
                     (void **)&p->d_bn, (void **)&p->d_rn, (void **)&p->d_part, (void **)&p->d_ir,
                     (void **)&p->d_cnt, &p->d_ell_val, &p->d_tcplanes, &p->d_tctab};
    for (void **b : bufs) {
        if (*b) cudaFree(*b);
        *b = nullptr;
    }
    p->bytes -= p->factor_bytes;
    p->factor_bytes = 0;
    p->factor_elt = 0;
    p->shift_cap = 0;
    const size_t before = p->bytes;
    const size_t c = (size_t)cap;
    KORE_TRY(kore_alloc(p, &p->d_Dinv, c * p->f_stride() * elt));
    KORE_TRY(kore_alloc(p, &p->d_Gm, c * p->f_stride() * elt));
    KORE_TRY(kore_alloc(p, &p->d_Hm, c * p->f_stride() * elt));
    KORE_TRY(kore_alloc(p, &p->d_Dw, c * p->f_stride() * elt));
    KORE_TRY(kore_alloc(p, &p->d_LU, c * p->lu_stride() * elt));
    KORE_TRY(kore_alloc(p, &p->d_T, c * p->t_stride() * elt));
    KORE_TRY(kore_alloc(p, &p->d_zlo, c * p->np * elt));
    KORE_TRY(kore_alloc(p, &p->d_xlo, c * p->np * elt));
    KORE_TRY(kore_alloc(p, &p->d_flo, c * p->np * elt));
    KORE_TRY(kore_alloc(p, (void **)&p->d_rscale, c * p->np * sizeof(double)));
    KORE_TRY(kore_alloc(p, (void **)&p->d_piv, c * p->p_stride() * sizeof(int)));
    KORE_TRY(kore_alloc(p, (void **)&p->d_pidx, c * p->p_stride() * sizeof(int)));
    KORE_TRY(kore_alloc(p, (void **)&p->d_used, c * p->p_stride() * sizeof(int)));
    KORE_TRY(kore_alloc(p, (void **)&p->d_sigma, c * sizeof(double2)));
    KORE_TRY(kore_alloc(p, (void **)&p->d_minf, c * sizeof(double)));
    KORE_TRY(kore_alloc(p, (void **)&p->d_bb, c * p->np * sizeof(double2)));
    KORE_TRY(kore_alloc(p, (void **)&p->d_xb, c * p->np * sizeof(double2)));
    KORE_TRY(kore_alloc(p, (void **)&p->d_rb, c * p->np * sizeof(double2)));
    KORE_TRY(kore_alloc(p, (void **)&p->d_bn, c * sizeof(double)));
    KORE_TRY(kore_alloc(p, (void **)&p->d_rn, c * sizeof(double)));
    // per-CTA maxima of the residual products: (np / 64 + np / 8 + 2) CTAs at most, 2 each
    KORE_TRY(kore_alloc(p, (void **)&p->d_part, c * 2 * (size_t)(p->np / 64 + p->np / 8 + 1024) * sizeof(double)));
    KORE_TRY(kore_alloc(p, (void **)&p->d_ir, c * sizeof(IrState)));
    KORE_TRY(kore_alloc(p, (void **)&p->d_cnt, c * (size_t)p->sweep_stages() * p->K * sizeof(int)));
    KORE_TRY(kore_alloc(p, &p->d_ell_val, c * std::max<int64_t>(p->ell_stride(), 1) * elt));
    if (elt == sizeof(float2)) {
        int64_t pl = 0, tb = 0;
        kore_tc_level_bytes(p, cap, &pl, &tb);
        KORE_TRY(kore_alloc(p, &p->d_tcplanes, (size_t)pl));
        KORE_TRY(kore_alloc(p, &p->d_tctab, (size_t)tb));
    }
    KORE_CUDA_TRY(cudaMemset(p->d_LU, 0, c * p->lu_stride() * elt));
    KORE_CUDA_TRY(cudaMemset(p->d_piv, 0, c * p->p_stride() * sizeof(int)));
    KORE_CUDA_TRY(cudaMemset(p->d_pidx, 0xff, c * p->p_stride() * sizeof(int)));
    KORE_CUDA_TRY(cudaMemset(p->d_used, 0, c * p->p_stride() * sizeof(int)));
    KORE_CUDA_TRY(cudaMemset(p->d_ir, 0, c * sizeof(IrState)));
    p->factor_bytes = p->bytes - before;
    p->factor_elt = elt;
    p->shift_cap = cap;
    return KORE_OK;
}

}  // namespace

int kore_factor_impl(kore_plan *p, int nshift, const double *sigmas, int precision) {
    if (precision != KORE_PREC_FP64 && precision != KORE_PREC_MIXED) return KORE_EINVAL;
    if (nshift <= 0 || !sigmas) return KORE_EINVAL;
    const size_t elt = (precision == KORE_PREC_FP64) ? sizeof(double2) : sizeof(float2);
    p->factored = false;
    KORE_TRY(ensure_factor_storage(p, nshift, elt));
    p->prec = precision;
    p->nshift = nshift;
    p->fw_lo = 0;
    p->fw_n = nshift;
    p->sigmas.assign(nshift, mk(0.0, 0.0));
    for (int s = 0; s < nshift; ++s) p->sigmas[s] = mk(sigmas[2 * s], sigmas[2 * s + 1]);
    p->sigma_re = sigmas[0];
    p->sigma_im = sigmas[1];
    KORE_CUDA_TRY(cudaMemcpyAsync(p->d_sigma, p->sigmas.data(), nshift * sizeof(double2), cudaMemcpyHostToDevice,
                                  p->stream));
    const unsigned grid = std::min<unsigned>(kore_div_up(p->np, 256), 64u);
    std::vector<double> red((size_t)grid * nshift);
    double *d_red = p->d_part;   // scratch: grid x nshift doubles fit the residual partials buffer
    if (p->prof) KORE_TRY(kore_prof_mark(p, 1, true));
    int s;
    if (precision == KORE_PREC_FP64) {
        k_rowinfo<double2><<<dim3(grid, nshift), 256, 0, p->stream>>>(make_fv<double2>(p), d_red);
        if (p->ell_stride() > 0)
            k_ell_fill<double2><<<dim3(std::min<unsigned>(kore_div_up(p->ell_stride(), 256), 4096u), nshift), 256, 0,
                              p->stream>>>(p->ell_stride(), p->ell_w, (p->S + 31) / 32, p->S, p->np, p->d_ell_src,
                                           p->d_aval, p->d_rscale, static_cast<double2 *>(p->d_ell_val));
        KORE_LAUNCHED(2);
        KORE_CUDA_TRY(cudaMemcpyAsync(red.data(), d_red, red.size() * sizeof(double), cudaMemcpyDeviceToHost, p->stream));
        KORE_CUDA_TRY(cudaStreamSynchronize(p->stream));
        s = factor_dispatch<double2>(p);
    } else {
        k_rowinfo<float2><<<dim3(grid, nshift), 256, 0, p->stream>>>(make_fv<float2>(p), d_red);
        if (p->ell_stride() > 0)
            k_ell_fill<float2><<<dim3(std::min<unsigned>(kore_div_up(p->ell_stride(), 256), 4096u), nshift), 256, 0,
                              p->stream>>>(p->ell_stride(), p->ell_w, (p->S + 31) / 32, p->S, p->np, p->d_ell_src,
                                           p->d_aval, p->d_rscale, static_cast<float2 *>(p->d_ell_val));
        KORE_LAUNCHED(2);
        KORE_CUDA_TRY(cudaMemcpyAsync(red.data(), d_red, red.size() * sizeof(double), cudaMemcpyDeviceToHost, p->stream));
        KORE_CUDA_TRY(cudaStreamSynchronize(p->stream));
        s = factor_dispatch<float2>(p);
    }
    if (s != KORE_OK) return s;
    if (p->prof) KORE_TRY(kore_prof_mark(p, 1, false));
    p->minfs.assign(nshift, 0.0);
    for (int sh = 0; sh < nshift; ++sh)
        for (unsigned b = 0; b < grid; ++b) p->minfs[sh] = std::max(p->minfs[sh], red[(size_t)sh * grid + b]);
    p->minf = p->minfs[0];
    KORE_CUDA_TRY(cudaMemcpyAsync(p->d_minf, p->minfs.data(), nshift * sizeof(double), cudaMemcpyHostToDevice,
                                  p->stream));
    KORE_CUDA_TRY(cudaStreamSynchronize(p->stream));
    KORE_TRY(kore_check_device_error(p));
    p->factored = true;
    return KORE_OK;
}

// Re-factorise one shift of a factorised plan: shift `slot` becomes A - sigma B and the
// other shifts keep their factors (the factor window is narrowed to the slot for the
// launches).  A batched eigensolve uses it to start a new target in a slot whose target
// has finished while the other slots carry on.
int kore_factor_slot(kore_plan *p, int slot, double sigma_re, double sigma_im) {
    if (!p->factored || slot < 0 || slot >= p->nshift) return KORE_EINVAL;
    p->factored = false;
    p->sigmas[slot] = mk(sigma_re, sigma_im);
    if (slot == 0) { p->sigma_re = sigma_re; p->sigma_im = sigma_im; }
    KORE_CUDA_TRY(cudaMemcpyAsync(p->d_sigma + slot, &p->sigmas[slot], sizeof(double2), cudaMemcpyHostToDevice,
                                  p->stream));
    p->fw_lo = slot;
    p->fw_n = 1;
    const unsigned grid = std::min<unsigned>(kore_div_up(p->np, 256), 64u);
    std::vector<double> red(grid);
    double *d_red = p->d_part;
    if (p->prof) KORE_TRY(kore_prof_mark(p, 1, true));
    int s;
    if (p->prec == KORE_PREC_FP64) {
        k_rowinfo<double2><<<dim3(grid, 1), 256, 0, p->stream>>>(make_fv<double2>(p), d_red);
        if (p->ell_stride() > 0)
            k_ell_fill<double2><<<dim3(std::min<unsigned>(kore_div_up(p->ell_stride(), 256), 4096u), 1), 256, 0,
                              p->stream>>>(p->ell_stride(), p->ell_w, (p->S + 31) / 32, p->S, p->np, p->d_ell_src,
                                           p->d_aval, p->d_rscale + (int64_t)slot * p->np,
                                           static_cast<double2 *>(p->d_ell_val) + (int64_t)slot * p->ell_stride());
        KORE_LAUNCHED(2);
        s = factor_dispatch<double2>(p);
    } else {
        k_rowinfo<float2><<<dim3(grid, 1), 256, 0, p->stream>>>(make_fv<float2>(p), d_red);
        if (p->ell_stride() > 0)
            k_ell_fill<float2><<<dim3(std::min<unsigned>(kore_div_up(p->ell_stride(), 256), 4096u), 1), 256, 0,
                              p->stream>>>(p->ell_stride(), p->ell_w, (p->S + 31) / 32, p->S, p->np, p->d_ell_src,
                                           p->d_aval, p->d_rscale + (int64_t)slot * p->np,
                                           static_cast<float2 *>(p->d_ell_val) + (int64_t)slot * p->ell_stride());
        KORE_LAUNCHED(2);
        s = factor_dispatch<float2>(p);
    }
    p->fw_lo = 0;
    p->fw_n = p->nshift;
    if (s != KORE_OK) return s;
    if (p->prof) KORE_TRY(kore_prof_mark(p, 1, false));
    KORE_CUDA_TRY(cudaMemcpyAsync(red.data(), d_red, red.size() * sizeof(double), cudaMemcpyDeviceToHost, p->stream));
    KORE_CUDA_TRY(cudaStreamSynchronize(p->stream));
    double mx = 0.0;
    for (unsigned b = 0; b < grid; ++b) mx = std::max(mx, red[b]);
    p->minfs[slot] = mx;
    if (slot == 0) p->minf = mx;
    KORE_CUDA_TRY(cudaMemcpyAsync(p->d_minf + slot, &p->minfs[slot], sizeof(double), cudaMemcpyHostToDevice,
                                  p->stream));
    KORE_CUDA_TRY(cudaStreamSynchronize(p->stream));
    KORE_TRY(kore_check_device_error(p));
    p->factored = true;
    return KORE_OK;
}

int kore_factor_reserve(kore_plan *p, int nslot, int precision) {
    if (nslot <= 0 || (precision != KORE_PREC_FP64 && precision != KORE_PREC_MIXED)) return KORE_EINVAL;
    const size_t elt = (precision == KORE_PREC_FP64) ? sizeof(double2) : sizeof(float2);
    p->factored = false;
    KORE_TRY(ensure_factor_storage(p, nslot, elt));
    p->prec = precision;
    p->nshift = nslot;
    p->fw_lo = 0;
    p->fw_n = nslot;
    // no slot holds a shift yet (NaN matches no target)
    p->sigmas.assign(nslot, mk(NAN, NAN));
    p->minfs.assign(nslot, 0.0);
    p->sigma_re = p->sigma_im = NAN;
    KORE_CUDA_TRY(cudaMemcpyAsync(p->d_sigma, p->sigmas.data(), nslot * sizeof(double2), cudaMemcpyHostToDevice,
                                  p->stream));
    KORE_CUDA_TRY(cudaMemcpyAsync(p->d_minf, p->minfs.data(), nslot * sizeof(double), cudaMemcpyHostToDevice,
                                  p->stream));
    KORE_CUDA_TRY(cudaStreamSynchronize(p->stream));
    p->factored = true;   // slot by slot from here (kore_factor_slot)
    return KORE_OK;
}
