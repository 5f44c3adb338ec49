// Block-Thomas factorisation of A - sigma*B over the l-major blocks.
//
// With D_i, L_i, U_i the diagonal, sub- and super-diagonal blocks of the (row
// equilibrated) l-major pencil R(A - sigma B), block Thomas forms the Schur
// complements S_0 = D_0, S_i = D_i - L_i X_{i-1}, where X_i = S_i^-1 U_i.  Each S_i is
// eliminated by Gauss-Jordan with partial pivoting on the augmented matrix
//     T = [ S_i | U_i | L_i | I ]          (S x 4S, column-major)
// which yields in one pass  X_i = S_i^-1 U_i,  W_i = S_i^-1 L_i  and  S_i^-1.
// The sweeps then need only dense matrix-vector products:
//     z_i = S_i^-1 c_i (all blocks at once),  y_i = z_i - W_i y_{i-1},  x_i = y_i - X_i x_{i+1}.
//
// The elimination is blocked: a panel of NB columns is reduced by one CTA in shared
// memory (pivot search over the rows not yet used, in-place Gauss-Jordan that turns
// the panel into the columns of the accumulated elementary transform E), then every
// trailing column t of T is updated by t <- E t, i.e. t[r] += sum_c E[r,c] t[piv_c]
// with the pivot rows themselves replaced.  Row swaps are never performed: the pivot
// row of column k is recorded and the outputs are gathered by it at the end.
//
// This is the arithmetic of the sparse LU that SLEPc's ST sinvert / PETSc's PCLU run
// inside bin/solve.py:123 and :227, restricted to the block-tridiagonal structure of
// the l-major pencil (no pivoting across blocks).
#include "kore_internal.cuh"
#include <climits>

namespace {

// Row equilibration by powers of two (exact): rscale[p] = 2^-e with
// e = exponent of max(max_e |a_pe|, |sigma| max_e |b_pe|); also the row 1-norms of
// |A| + |sigma||B| whose maximum is ||A - sigma B||_inf (upper bound).
__global__ void k_rowinfo(int64_t np, const int *__restrict__ arow, const double2 *__restrict__ aval,
                          const int *__restrict__ brow, const double *__restrict__ bval, int has_b,
                          double sabs, double *__restrict__ rscale, double *__restrict__ red) {
    double mx = 0.0;
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < np;
         p += (int64_t)gridDim.x * blockDim.x) {
        double am = 0.0, sum = 0.0;
        for (int e = arow[p]; e < arow[p + 1]; ++e) {
            double v = sqrt(abs2(aval[e]));
            am = fmax(am, v);
            sum += v;
        }
        if (has_b)
            for (int e = brow[p]; e < brow[p + 1]; ++e) {
                double v = sabs * fabs(bval[e]);
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

// T <- [0 | 0 | 0 | I] plus identity on the padded diagonal of the left block.
template <typename C>
__global__ void k_T_init(C *__restrict__ T, int S, int si) {
    const int64_t total = (int64_t)S * 4 * S;
    for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const int r = (int)(idx % S);
        const int64_t col = idx / S;
        C v = czero<C>();
        if (col == 3 * (int64_t)S + r || (col == r && r >= si)) v = cone<C>();
        T[idx] = v;
    }
}

// Scatter row k of block i: D_i - sigma B_i into T[:,0:S), U_i into T[:,S:2S),
// L_i into T[:,2S:3S), all times the row scale.  A and B rows are merged by column
// so that each entry of D - sigma B is formed in FP64 and rounded once.
template <typename C>
__global__ void k_T_scatter(C *__restrict__ T, int S, int i, int si, const int *__restrict__ arow,
                            const int *__restrict__ acol, const double2 *__restrict__ aval,
                            const int *__restrict__ asplit, const int *__restrict__ brow,
                            const int *__restrict__ bcol, const double *__restrict__ bval, int has_b,
                            double sre, double sim, const double *__restrict__ rscale) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= si) return;
    const double2 sigma = mk(sre, sim);
    const int64_t p = (int64_t)i * S + k;
    const double rs = rscale[p];
    const int e0 = arow[p], eD = asplit[2 * p], eU = asplit[2 * p + 1], e1 = arow[p + 1];
    const int64_t base = (int64_t)i * S;
    for (int e = e0; e < eD; ++e) {
        const int c = (int)(acol[e] - (base - S));
        T[k + (int64_t)(2 * S + c) * S] = from_c128<C>(rs * aval[e]);
    }
    int ea = eD, eb = has_b ? brow[p] : 0;
    const int eb1 = has_b ? brow[p + 1] : 0;
    while (ea < eU || eb < eb1) {
        const int ca = (ea < eU) ? acol[ea] : INT_MAX;
        const int cb = (eb < eb1) ? bcol[eb] : INT_MAX;
        const int c = min(ca, cb);
        double2 v = mk(0.0, 0.0);
        if (ca == c) { v = aval[ea]; ++ea; }
        if (cb == c) { v = v - bval[eb] * sigma; ++eb; }
        T[k + (int64_t)(c - base) * S] = from_c128<C>(rs * v);
    }
    for (int e = eU; e < e1; ++e) {
        const int c = (int)(acol[e] - (base + S));
        T[k + (int64_t)(S + c) * S] = from_c128<C>(rs * aval[e]);
    }
}

// Schur complement: T[k, j] -= sum_{e in L_i(k)} rs * a_e * X_{i-1}[c_e, j], j < S.
template <typename C>
__global__ void k_T_schur(C *__restrict__ T, int S, int i, const int *__restrict__ arow,
                          const int *__restrict__ acol, const double2 *__restrict__ aval,
                          const int *__restrict__ asplit, const double *__restrict__ rscale,
                          const C *__restrict__ Xprev) {
    const int k = blockIdx.x;
    const int64_t p = (int64_t)i * S + k;
    const int e0 = arow[p], eD = asplit[2 * p];
    if (e0 == eD) return;
    const double rs = rscale[p];
    const int64_t base_prev = (int64_t)(i - 1) * S;
    for (int j = threadIdx.x; j < S; j += blockDim.x) {
        C acc = czero<C>();
        for (int e = e0; e < eD; ++e) {
            const int c = (int)(acol[e] - base_prev);
            acc = cfma(acc, from_c128<C>(rs * aval[e]), Xprev[(int64_t)c * S + j]);
        }
        const int64_t idx = k + (int64_t)j * S;
        T[idx] = T[idx] - acc;
    }
}

// Panel reduction of columns [k0, k0+nb) of T by one CTA (see file header).
template <typename C, int NB>
__global__ void __launch_bounds__(512) k_panel(C *__restrict__ T, int S, int k0, int *__restrict__ piv,
                                               int *__restrict__ pidx, int *__restrict__ used,
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
    const int tid = threadIdx.x, nt = blockDim.x;
    const int nb = min(NB, S - k0);

    for (int idx = tid; idx < S * nb; idx += nt) P[idx] = T[(int64_t)k0 * S + idx];
    for (int r = tid; r < S; r += nt) u[r] = used[r];
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
        for (int o = 16; o > 0; o >>= 1) {
            const double ov = __shfl_down_sync(0xffffffffu, best, o);
            const int oi = __shfl_down_sync(0xffffffffu, bi, o);
            if (ov > best || (ov == best && oi < bi)) { best = ov; bi = oi; }
        }
        if ((tid & 31) == 0) { rv[tid >> 5] = best; ri[tid >> 5] = bi; }
        __syncthreads();
        if (tid < 32) {
            const int nw = nt >> 5;
            best = (tid < nw) ? rv[tid] : -1.0;
            bi = (tid < nw) ? ri[tid] : INT_MAX;
            for (int o = 16; o > 0; o >>= 1) {
                const double ov = __shfl_down_sync(0xffffffffu, best, o);
                const int oi = __shfl_down_sync(0xffffffffu, bi, o);
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
        for (int idx = tid; idx < S * nb; idx += nt) {
            const int cc = idx / S, r = idx - cc * S;
            if (cc == c) continue;
            P[idx] = (r == p) ? prow[cc] : cfms(P[idx], P[c * S + r], prow[cc]);
        }
        __syncthreads();
        for (int r = tid; r < S; r += nt) P[c * S + r] = (r == p) ? dinv : -(P[c * S + r] * dinv);
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

// Trailing update of TW columns per CTA: t <- E t for the panel at k0.
template <typename C, int NB, int TW>
__global__ void __launch_bounds__(256) k_update(C *__restrict__ T, int S, int k0, int nb, int col_begin,
                                                int col_end, const int *__restrict__ piv,
                                                const int *__restrict__ pidx) {
    __shared__ C tp[TW][NB];
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
#pragma unroll
        for (int t = 0; t < TW; ++t) {
            if (t < tw) {
                const int64_t idx = r + (int64_t)(j0 + t) * S;
                C acc = isp ? czero<C>() : T[idx];
#pragma unroll
                for (int c = 0; c < NB; ++c) acc = cfma(acc, er[c], tp[t][c]);
                T[idx] = acc;
            }
        }
    }
}

// Gather the solution rows by pivot: Sinv[k,:] = T[piv[k], 3S:4S), W[k,:] from
// T[:, 2S:3S), X[k,:] from T[:, S:2S)  (row-major S x S blocks).
template <typename C>
__global__ void k_extract(const C *__restrict__ T, int S, const int *__restrict__ piv, C *__restrict__ Sinv,
                          C *__restrict__ W, C *__restrict__ X, int has_prev, int has_next) {
    const int64_t total = (int64_t)S * S;
    for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const int k = (int)(idx / S), j = (int)(idx - (int64_t)k * S);
        const int p = piv[k];
        Sinv[idx] = T[p + (int64_t)(3 * S + j) * S];
        W[idx] = has_prev ? T[p + (int64_t)(2 * S + j) * S] : czero<C>();
        X[idx] = has_next ? T[p + (int64_t)(S + j) * S] : czero<C>();
    }
}

constexpr int kUpdTW = 8;

template <typename C, int NB>
int factor_blocks(kore_plan *p) {
    const int S = p->S, K = p->K;
    C *T = static_cast<C *>(p->d_T);
    C *Sinv = static_cast<C *>(p->d_sinv), *W = static_cast<C *>(p->d_W), *X = static_cast<C *>(p->d_X);
    const int64_t SS = (int64_t)S * S;
    const size_t smem = (size_t)S * NB * sizeof(C) + (size_t)S * sizeof(int);
    KORE_CUDA_TRY(cudaFuncSetAttribute(k_panel<C, NB>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    cudaStream_t st = p->stream;
    const unsigned initGrid = std::min<unsigned>(kore_div_up((int64_t)S * 4 * S, 256), 8u * p->num_sms);
    const unsigned exGrid = std::min<unsigned>(kore_div_up(SS, 256), 8u * p->num_sms);
    for (int i = 0; i < K; ++i) {
        const int si = p->bsz[i];
        k_T_init<C><<<initGrid, 256, 0, st>>>(T, S, si);
        k_T_scatter<C><<<kore_div_up(si, 128), 128, 0, st>>>(
            T, S, i, si, p->d_arow, p->d_acol, p->d_aval, p->d_asplit, p->d_brow, p->d_bcol, p->d_bval,
            p->has_b ? 1 : 0, p->sigma_re, p->sigma_im, p->d_rscale);
        KORE_LAUNCHED(2);
        if (i > 0) {
            k_T_schur<C><<<si, 128, 0, st>>>(T, S, i, p->d_arow, p->d_acol, p->d_aval, p->d_asplit,
                                             p->d_rscale, X + (int64_t)(i - 1) * SS);
            KORE_LAUNCHED(1);
        }
        KORE_CUDA_TRY(cudaMemsetAsync(p->d_used, 0, sizeof(int) * S, st));
        for (int k0 = 0; k0 < S; k0 += NB) {
            const int nb = std::min(NB, S - k0);
            k_panel<C, NB><<<1, 512, smem, st>>>(T, S, k0, p->d_piv, p->d_pidx, p->d_used, p->d_err);
            const int cb = k0 + nb, ce = 4 * S;
            k_update<C, NB, kUpdTW><<<kore_div_up(ce - cb, kUpdTW), 256, 0, st>>>(T, S, k0, nb, cb, ce,
                                                                                 p->d_piv, p->d_pidx);
            KORE_LAUNCHED(2);
        }
        k_extract<C><<<exGrid, 256, 0, st>>>(T, S, p->d_piv, Sinv + i * SS, W + i * SS, X + i * SS,
                                             i > 0 ? 1 : 0, i + 1 < K ? 1 : 0);
        KORE_LAUNCHED(1);
        KORE_CUDA_TRY(cudaGetLastError());
    }
    return KORE_OK;
}

template <typename C>
int factor_dispatch(kore_plan *p) {
    // widest panel that fits the 227 KB shared-memory limit
    const size_t cap = 220 * 1024;
    auto fits = [&](int nb) { return (size_t)p->S * nb * sizeof(C) + (size_t)p->S * sizeof(int) <= cap; };
    if (sizeof(C) == 8 && fits(32)) return factor_blocks<C, 32>(p);
    if (fits(16)) return factor_blocks<C, 16>(p);
    if (fits(8)) return factor_blocks<C, 8>(p);
    if (fits(4)) return factor_blocks<C, 4>(p);
    return KORE_EINVAL;
}

}  // namespace

int kore_factor_impl(kore_plan *p, double sre, double sim, int precision) {
    if (precision != KORE_PREC_FP64 && precision != KORE_PREC_MIXED) return KORE_EINVAL;
    const size_t elt = (precision == KORE_PREC_FP64) ? sizeof(double2) : sizeof(float2);
    const int64_t SS = (int64_t)p->S * p->S;
    if (p->factor_elt != elt) {
        cudaFree(p->d_sinv); cudaFree(p->d_W); cudaFree(p->d_X); cudaFree(p->d_T);
        cudaFree(p->d_zlo); cudaFree(p->d_ylo);
        p->d_sinv = p->d_W = p->d_X = p->d_T = p->d_zlo = p->d_ylo = nullptr;
        if (p->factor_elt) p->bytes -= (3 * (size_t)p->K * SS + 4 * (size_t)SS + 2 * (size_t)p->np) * p->factor_elt;
        p->factor_elt = 0;
        KORE_TRY(kore_alloc(p, &p->d_sinv, (size_t)p->K * SS * elt));
        KORE_TRY(kore_alloc(p, &p->d_W, (size_t)p->K * SS * elt));
        KORE_TRY(kore_alloc(p, &p->d_X, (size_t)p->K * SS * elt));
        KORE_TRY(kore_alloc(p, &p->d_T, (size_t)4 * SS * elt));
        KORE_TRY(kore_alloc(p, &p->d_zlo, (size_t)p->np * elt));
        KORE_TRY(kore_alloc(p, &p->d_ylo, (size_t)p->np * elt));
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
