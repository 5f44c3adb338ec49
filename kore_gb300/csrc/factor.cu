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
// This replaces the sparse LU that SLEPc's ST sinvert / PETSc's PCLU build inside
// bin/solve.py:123 and :227; the ordering (odd-even elimination of l-blocks) is what
// exposes the parallelism.
#include "kore_internal.cuh"
#include <climits>
#include <algorithm>

namespace {

// Row equilibration by powers of two (exact): rscale[p] = 2^-e with
// e = exponent of max(max_e |a_pe|, |sigma| max_e |b_pe|); also the row 1-norms of
// |A| + |sigma||B| whose maximum bounds ||A - sigma B||_inf.
__global__ void k_rowinfo(int64_t np, const int *__restrict__ arow, const double2 *__restrict__ aval,
                          const int *__restrict__ brow, const double *__restrict__ bval, int has_b,
                          double sabs, double *__restrict__ rscale, double *__restrict__ red) {
    double mx = 0.0;
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < np;
         p += (int64_t)gridDim.x * blockDim.x) {
        double am = 0.0, sum = 0.0;
        for (int e = arow[p]; e < arow[p + 1]; ++e) {
            const double v = sqrt(abs2(aval[e]));
            am = fmax(am, v);
            sum += v;
        }
        if (has_b)
            for (int e = brow[p]; e < brow[p + 1]; ++e) {
                const double v = sabs * fabs(bval[e]);
                am = fmax(am, v);
                sum += v;
            }
        rscale[p] = (am > 0.0) ? ldexp(1.0, -ilogb(am)) : 1.0;
        mx = fmax(mx, sum);
    }
    mx = warp_max_d(mx);
    __shared__ double sm[32];
    if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = mx;
    __syncthreads();
    if (threadIdx.x < 32) {
        double v = (threadIdx.x < (blockDim.x >> 5)) ? sm[threadIdx.x] : 0.0;
        v = warp_max_d(v);
        if (threadIdx.x == 0) red[blockIdx.x] = v;
    }
}

// Dw <- 0 with the identity on the padded diagonal of every block.
template <typename C>
__global__ void k_Dw_init(C *__restrict__ Dw, int K, int S, const int *__restrict__ bsz) {
    const int64_t SS = (int64_t)S * S, total = (int64_t)K * SS;
    for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = idx / SS;
        const int64_t e = idx - i * SS;
        const int c = (int)(e / S), r = (int)(e - (int64_t)c * S);
        Dw[idx] = (r == c && r >= bsz[i]) ? cone<C>() : czero<C>();
    }
}

// One warp per row: Dw_i[r, :] = rs_r (D_i - sigma B_i)[r, :] from the CSR.  A and B
// entries of the same column are combined in FP64 and rounded once.
template <typename C>
__global__ void k_Dw_scatter(C *__restrict__ Dw, int64_t np, int S, const int *__restrict__ arow,
                             const int *__restrict__ acol, const double2 *__restrict__ aval,
                             const int *__restrict__ asplit, const int *__restrict__ brow,
                             const int *__restrict__ bcol, const double *__restrict__ bval, int has_b,
                             double sre, double sim, const double *__restrict__ rscale) {
    const int lane = threadIdx.x & 31;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const double2 sigma = mk(sre, sim);
    for (int64_t p = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5; p < np; p += nw) {
        const int64_t i = p / S;
        const int r = (int)(p - i * S);
        const double rs = rscale[p];
        C *D = Dw + i * (int64_t)S * S;
        const int eD = asplit[2 * p], eU = asplit[2 * p + 1];
        for (int e = eD + lane; e < eU; e += 32) D[r + (int64_t)(acol[e] - i * S) * S] = from_c128<C>(rs * aval[e]);
        __syncwarp();
        if (has_b)
            for (int e = brow[p] + lane; e < brow[p + 1]; e += 32) {
                const int c = bcol[e];
                // matching A entry (binary search in the sorted D segment)
                int lo = eD, hi = eU;
                while (lo < hi) {
                    const int mid = (lo + hi) >> 1;
                    if (acol[mid] < c) lo = mid + 1; else hi = mid;
                }
                const double2 a = (lo < eU && acol[lo] == c) ? aval[lo] : mk(0.0, 0.0);
                D[r + (int64_t)(c - i * S) * S] = from_c128<C>(rs * (a - bval[e] * sigma));
            }
    }
}

// T_o = [Dw_j | L | U | I] for the odd blocks j of level lv; L, U copied from the
// dense couplings (levels >= 1) or zeroed (level 0: scattered from the CSR next).
// stride 0 selects block 0 (the top of the reduction).
template <typename C>
__global__ void k_T_fill(C *__restrict__ T, const C *__restrict__ Dw, const C *__restrict__ LU, int S,
                         BcrLevel lv, int nodd) {
    const int64_t SS = (int64_t)S * S, per = 4 * SS, total = (int64_t)nodd * per;
    for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const int64_t o = idx / per;
        const int64_t e = idx - o * per;
        const int part = (int)(e / SS);
        const int64_t w = e - (int64_t)part * SS;
        const int64_t q = 2 * o + 1;               // position of the odd block
        const int64_t j = q * lv.stride;           // original block
        C v;
        if (part == 0) v = Dw[j * SS + w];
        else if (part == 3) {
            const int c = (int)(w / S), r = (int)(w - (int64_t)c * S);
            v = (r == c) ? cone<C>() : czero<C>();
        } else if (lv.lu_L < 0) v = czero<C>();
        else v = LU[((part == 1 ? lv.lu_L : lv.lu_U) + q) * SS + w];
        T[idx] = v;
    }
}

// Level 0: one warp per row of an odd block j: scatter rs * L_j and rs * U_j into T_o.
template <typename C>
__global__ void k_T_scatter_LU(C *__restrict__ T, int S, int nodd, const int *__restrict__ arow,
                               const int *__restrict__ acol, const double2 *__restrict__ aval,
                               const int *__restrict__ asplit, const double *__restrict__ rscale) {
    const int lane = threadIdx.x & 31;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const int64_t SS = (int64_t)S * S;
    for (int64_t w = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5; w < (int64_t)nodd * S; w += nw) {
        const int64_t o = w / S;
        const int r = (int)(w - o * S);
        const int64_t j = 2 * o + 1;
        const int64_t p = j * S + r;
        const double rs = rscale[p];
        C *To = T + o * 4 * SS;
        for (int e = arow[p] + lane; e < asplit[2 * p]; e += 32)
            To[r + (int64_t)(S + acol[e] - (j - 1) * S) * S] = from_c128<C>(rs * aval[e]);
        for (int e = asplit[2 * p + 1] + lane; e < arow[p + 1]; e += 32)
            To[r + (int64_t)(2 * S + acol[e] - (j + 1) * S) * S] = from_c128<C>(rs * aval[e]);
    }
}

// Panel reduction of columns [k0, k0+nb) of T_o, one CTA per odd block o.
template <typename C, int NB>
__global__ void __launch_bounds__(1024) k_panel(C *__restrict__ Tall, int S, int k0, int *__restrict__ pivall,
                                                int *__restrict__ pidxall, int *__restrict__ usedall,
                                                int *__restrict__ err) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    C *P = reinterpret_cast<C *>(smem_raw);
    int *u = reinterpret_cast<int *>(P + (size_t)S * NB);
    __shared__ C prow[NB];
    __shared__ double rv[32];
    __shared__ int ri[32];
    __shared__ int s_p;
    __shared__ C s_dinv;
    __shared__ int s_piv[NB];
    const int64_t o = blockIdx.x;
    C *T = Tall + o * 4 * (int64_t)S * S;
    int *piv = pivall + o * S, *pidx = pidxall + o * S, *used = usedall + o * S;
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
                const double v = (double)abs2(P[c * S + r]);
                if (v > best) { best = v; bi = r; }
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
                    atomicCAS(err, 0, KORE_DEVERR_PIVOT);
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

// Trailing update of TW columns per CTA (blockIdx.x) of odd block blockIdx.y.
template <typename C, int NB, int TW>
__global__ void __launch_bounds__(256) k_update(C *__restrict__ Tall, int S, int k0, int nb, int col_begin,
                                                int col_end, const int *__restrict__ pivall,
                                                const int *__restrict__ pidxall) {
    __shared__ C tp[TW][NB];
    const int64_t o = blockIdx.y;
    C *T = Tall + o * 4 * (int64_t)S * S;
    const int *piv = pivall + o * S, *pidx = pidxall + o * S;
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

// Solution rows by pivot: Dinv_j[k,:] = T[piv[k], 3S:4S), G_j from T[:, S:2S),
// H_j from T[:, 2S:3S)  (column-major S x S outputs).
template <typename C>
__global__ void k_extract(const C *__restrict__ Tall, int S, const int *__restrict__ pivall, C *__restrict__ Dinv,
                          C *__restrict__ G, C *__restrict__ H, BcrLevel lv, int nodd, int top) {
    const int64_t SS = (int64_t)S * S, total = (int64_t)nodd * SS;
    for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const int64_t o = idx / SS;
        const int64_t w = idx - o * SS;
        const int c = (int)(w / S), k = (int)(w - (int64_t)c * S);
        const C *T = Tall + o * 4 * SS;
        const int p = pivall[o * S + k];
        const int64_t j = top ? 0 : (2 * o + 1) * lv.stride;
        Dinv[j * SS + w] = T[p + (int64_t)(3 * S + c) * S];
        if (!top) {
            G[j * SS + w] = T[p + (int64_t)(S + c) * S];
            H[j * SS + w] = T[p + (int64_t)(2 * S + c) * S];
        }
    }
}

// Level 0 update of the even blocks with the sparse couplings of the CSR:
//   Dw_i -= rs (L_i H_jl + U_i G_jr),  L'_i = -rs L_i G_jl,  U'_i = -rs U_i H_jr.
// CTA = (chunk of CW columns, even index e); one thread per row.
constexpr int kEvenCW = 8;
template <typename C>
__global__ void k_even_l0(C *__restrict__ Dw, C *__restrict__ LU, const C *__restrict__ G, const C *__restrict__ H,
                          int S, BcrLevel lv, const int *__restrict__ arow, const int *__restrict__ acol,
                          const double2 *__restrict__ aval, const int *__restrict__ asplit,
                          const double *__restrict__ rscale) {
    const int64_t SS = (int64_t)S * S;
    const int64_t e = blockIdx.y;
    const int64_t q = 2 * e;                 // position = original block at level 0
    const bool hasl = q >= 1, hasr = q + 1 < lv.Kl;
    const bool outl = (lv.lu_nL >= 0) && q >= 2, outr = (lv.lu_nU >= 0) && q + 2 < lv.Kl;
    const int c0 = blockIdx.x * kEvenCW;
    const int cn = min(kEvenCW, S - c0);
    C *Di = Dw + q * SS;
    for (int r = threadIdx.x; r < S; r += blockDim.x) {
        const int64_t p = q * S + r;
        const int l0 = arow[p], l1 = asplit[2 * p], u0 = asplit[2 * p + 1], u1 = arow[p + 1];
        const double rs = rscale[p];
        for (int t = 0; t < cn; ++t) {
            const int64_t col = (int64_t)(c0 + t) * S;
            C dsum = czero<C>(), lsum = czero<C>(), usum = czero<C>();
            if (hasl)
                for (int k = l0; k < l1; ++k) {
                    const C a = from_c128<C>(rs * aval[k]);
                    const int64_t cr = acol[k] - (q - 1) * S;
                    dsum = cfma(dsum, a, H[(q - 1) * SS + cr + col]);
                    if (outl) lsum = cfma(lsum, a, G[(q - 1) * SS + cr + col]);
                }
            if (hasr)
                for (int k = u0; k < u1; ++k) {
                    const C a = from_c128<C>(rs * aval[k]);
                    const int64_t cr = acol[k] - (q + 1) * S;
                    dsum = cfma(dsum, a, G[(q + 1) * SS + cr + col]);
                    if (outr) usum = cfma(usum, a, H[(q + 1) * SS + cr + col]);
                }
            Di[r + col] = Di[r + col] - dsum;
            if (outl) LU[(lv.lu_nL + e) * SS + r + col] = -lsum;
            if (outr) LU[(lv.lu_nU + e) * SS + r + col] = -usum;
        }
    }
}

// Batched dense update of the even blocks at levels >= 1, one GEMM job per
// (even block, kind): kind 0: Dw_i -= L_q H_jl + U_q G_jr;  kind 1: L' = -L_q G_jl;
// kind 2: U' = -U_q H_jr.  Column-major S x S complex, 64 x 64 tiles, 4 x 4 per thread.
constexpr int kGT = 64, kGK = 16;
template <typename C>
__global__ void __launch_bounds__(256) k_even_gemm(C *__restrict__ Dw, C *__restrict__ LU, const C *__restrict__ G,
                                                   const C *__restrict__ H, int S, BcrLevel lv) {
    __shared__ C As[kGK][kGT + 1];
    __shared__ C Bs[kGK][kGT + 1];
    const int64_t SS = (int64_t)S * S;
    const int job = blockIdx.z;
    const int64_t e = job / 3;
    const int kind = job - 3 * (int)e;
    const int64_t q = 2 * e;
    const bool hasl = q >= 1, hasr = q + 1 < lv.Kl;
    const C *A1 = nullptr, *B1 = nullptr, *A2 = nullptr, *B2 = nullptr;
    C *Cm = nullptr;
    bool accumulate = false;
    const C *Lq = LU + (lv.lu_L + q) * SS, *Uq = LU + (lv.lu_U + q) * SS;
    const int64_t jl = (q - 1) * lv.stride, jr = (q + 1) * lv.stride;
    if (kind == 0) {
        Cm = Dw + q * lv.stride * SS;
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
    const int m0 = blockIdx.x * kGT, n0 = blockIdx.y * kGT;
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;   // 16 x 16 threads, 4 x 4 each
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
                Cm[idx] = accumulate ? Cm[idx] - acc[a][b] : -acc[a][b];
            }
        }
}

constexpr int kUpdTW = 8;

unsigned grid_for(int64_t work, int threads, int num_sms) {
    return (unsigned)std::max<int64_t>(1, std::min<int64_t>((work + threads - 1) / threads, 16LL * num_sms));
}

// Gauss-Jordan of the nodd work matrices T_o (all panels), then extraction.
template <typename C, int NB>
int gauss_jordan(kore_plan *p, const BcrLevel &lv, int nodd, int top) {
    const int S = p->S;
    C *T = static_cast<C *>(p->d_T);
    const size_t smem = (size_t)S * NB * sizeof(C) + (size_t)S * sizeof(int);
    KORE_CUDA_TRY(cudaFuncSetAttribute(k_panel<C, NB>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    const int pthreads = std::min(1024, ((S + 31) / 32) * 32);
    for (int k0 = 0; k0 < S; k0 += NB) {
        const int nb = std::min(NB, S - k0);
        k_panel<C, NB><<<nodd, pthreads, smem, p->stream>>>(T, S, k0, p->d_piv, p->d_pidx, p->d_used, p->d_err);
        KORE_LAUNCHED(1);
        const int cb = k0 + nb;
        if (!top) {
            // trailing columns: the rest of D, the L, U and identity columns
            dim3 g(kore_div_up(4 * S - cb, kUpdTW), nodd);
            k_update<C, NB, kUpdTW><<<g, 256, 0, p->stream>>>(T, S, k0, nb, cb, 4 * S, p->d_piv, p->d_pidx);
            KORE_LAUNCHED(1);
        } else {
            // the top block has no L, U columns: the rest of D, then the identity columns
            if (cb < S) {
                dim3 g(kore_div_up(S - cb, kUpdTW), nodd);
                k_update<C, NB, kUpdTW><<<g, 256, 0, p->stream>>>(T, S, k0, nb, cb, S, p->d_piv, p->d_pidx);
                KORE_LAUNCHED(1);
            }
            dim3 g(kore_div_up(S, kUpdTW), nodd);
            k_update<C, NB, kUpdTW><<<g, 256, 0, p->stream>>>(T, S, k0, nb, 3 * S, 4 * S, p->d_piv, p->d_pidx);
            KORE_LAUNCHED(1);
        }
    }
    k_extract<C><<<grid_for((int64_t)nodd * S * S, 256, p->num_sms), 256, 0, p->stream>>>(
        T, S, p->d_piv, static_cast<C *>(p->d_Dinv), static_cast<C *>(p->d_Gm), static_cast<C *>(p->d_Hm), lv,
        nodd, top);
    KORE_LAUNCHED(1);
    KORE_CUDA_TRY(cudaGetLastError());
    return KORE_OK;
}

template <typename C, int NB>
int factor_levels(kore_plan *p) {
    const int S = p->S, K = p->K;
    const int64_t SS = (int64_t)S * S;
    cudaStream_t st = p->stream;
    C *Dw = static_cast<C *>(p->d_Dw), *LU = static_cast<C *>(p->d_LU), *T = static_cast<C *>(p->d_T);
    C *G = static_cast<C *>(p->d_Gm), *H = static_cast<C *>(p->d_Hm);
    // working diagonal blocks from the CSR
    k_Dw_init<C><<<grid_for((int64_t)K * SS, 256, p->num_sms), 256, 0, st>>>(Dw, K, S, p->d_bsz);
    k_Dw_scatter<C><<<grid_for(p->np * 32, 256, p->num_sms), 256, 0, st>>>(
        Dw, p->np, S, p->d_arow, p->d_acol, p->d_aval, p->d_asplit, p->d_brow, p->d_bcol, p->d_bval,
        p->has_b ? 1 : 0, p->sigma_re, p->sigma_im, p->d_rscale);
    KORE_LAUNCHED(2);
    for (int l = 0; l < p->nlev; ++l) {
        const BcrLevel &lv = p->lev[l];
        k_T_fill<C><<<grid_for((int64_t)lv.nodd * 4 * SS, 256, p->num_sms), 256, 0, st>>>(T, Dw, LU, S, lv, lv.nodd);
        KORE_LAUNCHED(1);
        if (l == 0) {
            k_T_scatter_LU<C><<<grid_for((int64_t)lv.nodd * S * 32, 256, p->num_sms), 256, 0, st>>>(
                T, S, lv.nodd, p->d_arow, p->d_acol, p->d_aval, p->d_asplit, p->d_rscale);
            KORE_LAUNCHED(1);
        }
        KORE_TRY((gauss_jordan<C, NB>(p, lv, lv.nodd, 0)));
        if (l == 0) {
            dim3 g(kore_div_up(S, kEvenCW), lv.neven);
            const int th = std::min(1024, ((S + 31) / 32) * 32);
            k_even_l0<C><<<g, th, 0, st>>>(Dw, LU, G, H, S, lv, p->d_arow, p->d_acol, p->d_aval, p->d_asplit,
                                          p->d_rscale);
        } else {
            dim3 g(kore_div_up(S, kGT), kore_div_up(S, kGT), 3 * lv.neven);
            k_even_gemm<C><<<g, 256, 0, st>>>(Dw, LU, G, H, S, lv);
        }
        KORE_LAUNCHED(1);
        KORE_CUDA_TRY(cudaGetLastError());
    }
    // the last active block (block 0): T = [Dw_0 | 0 | 0 | I]; stride 0 maps odd index 0 to block 0
    BcrLevel top{};
    top.Kl = 1;
    top.stride = 0;
    top.lu_L = top.lu_U = top.lu_nL = top.lu_nU = -1;
    k_T_fill<C><<<grid_for(4 * SS, 256, p->num_sms), 256, 0, st>>>(T, Dw, LU, S, top, 1);
    KORE_LAUNCHED(1);
    KORE_TRY((gauss_jordan<C, NB>(p, top, 1, 1)));
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

int kore_factor_impl(kore_plan *p, double sre, double sim, int precision) {
    if (precision != KORE_PREC_FP64 && precision != KORE_PREC_MIXED) return KORE_EINVAL;
    const size_t elt = (precision == KORE_PREC_FP64) ? sizeof(double2) : sizeof(float2);
    const int64_t SS = (int64_t)p->S * p->S;
    if (p->factor_elt != elt) {
        void **bufs[] = {&p->d_Dinv, &p->d_Gm, &p->d_Hm, &p->d_Dw, &p->d_LU, &p->d_T, &p->d_zlo, &p->d_xlo, &p->d_flo};
        for (void **b : bufs) {
            if (*b) cudaFree(*b);
            *b = nullptr;
        }
        p->factor_elt = 0;
        KORE_TRY(kore_alloc(p, &p->d_Dinv, (size_t)p->K * SS * elt));
        KORE_TRY(kore_alloc(p, &p->d_Gm, (size_t)p->K * SS * elt));
        KORE_TRY(kore_alloc(p, &p->d_Hm, (size_t)p->K * SS * elt));
        KORE_TRY(kore_alloc(p, &p->d_Dw, (size_t)p->K * SS * elt));
        KORE_TRY(kore_alloc(p, &p->d_LU, (size_t)p->lu_mats * SS * elt));
        KORE_TRY(kore_alloc(p, &p->d_T, (size_t)p->nodd_max * 4 * SS * elt));
        KORE_TRY(kore_alloc(p, &p->d_zlo, (size_t)p->np * elt));
        KORE_TRY(kore_alloc(p, &p->d_xlo, (size_t)p->np * elt));
        KORE_TRY(kore_alloc(p, &p->d_flo, (size_t)p->np * elt));
        KORE_CUDA_TRY(cudaMemset(p->d_LU, 0, (size_t)p->lu_mats * SS * elt));
        p->factor_elt = elt;
    }
    p->factored = false;
    p->prec = precision;
    p->sigma_re = sre;
    p->sigma_im = sim;
    const unsigned grid = std::min<unsigned>(kore_div_up(p->np, 256), 1024u);
    k_rowinfo<<<grid, 256, 0, p->stream>>>(p->np, p->d_arow, p->d_aval, p->d_brow, p->d_bval,
                                           p->has_b ? 1 : 0, std::hypot(sre, sim), p->d_rscale, p->d_red);
    KORE_LAUNCHED(1);
    KORE_CUDA_TRY(cudaMemcpyAsync(p->h_red, p->d_red, grid * sizeof(double), cudaMemcpyDeviceToHost, p->stream));
    if (p->prof) KORE_TRY(kore_prof_mark(p, 1, true));
    int s = (precision == KORE_PREC_FP64) ? factor_dispatch<double2>(p) : factor_dispatch<float2>(p);
    if (s != KORE_OK) return s;
    if (p->prof) KORE_TRY(kore_prof_mark(p, 1, false));
    KORE_CUDA_TRY(cudaStreamSynchronize(p->stream));
    double mx = 0.0;
    for (unsigned b = 0; b < grid; ++b) mx = std::max(mx, p->h_red[b]);
    p->minf = mx;
    KORE_TRY(kore_check_device_error(p));
    p->factored = true;
    return KORE_OK;
}
