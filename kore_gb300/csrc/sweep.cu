// Solves with the block-cyclic-reduction factors of factor.cu, sparse products and
// the FP64 refinement loop.
//
// (A - sigma B) x = b with row scaling R and s = ||b||_inf (keeps complex64 in range):
// the right-hand side c = s^-1 R b is reduced level by level exactly as the blocks were,
//     level l, odd blocks j:   z_j = D_j^-1 f_j
//     level l, even blocks i:  f_i <- f_i - L_i z_jl - U_i z_jr        (CSR couplings at level 0)
// the last block is solved, x_0 = D_0^-1 f_0, and the levels are unwound in reverse,
//     level l, odd blocks j:   x_j = z_j - G_j x_jl - H_j x_jr,
// then x <- s x.  One cooperative persistent kernel runs all phases (about 3 log2 K of
// them) with a bounded grid barrier between dependent phases; inside a phase every
// (block, row tile) is independent, so each phase is a batched matrix-vector product
// streaming the factors from HBM across the whole GPU.
//
// In mixed precision the factors are complex64 and the result is refined in FP64:
//     r = b - (A - sigma B) x,  x += M32^-1 r   until ||r||_inf <= tol (||M||_inf ||x||_inf + ||b||_inf).
#include "kore_internal.cuh"
#include <cstddef>
#include <mutex>

namespace {

constexpr int kSweepWarps = 8;                 // warps of a sweep CTA; they split the columns
constexpr int kSweepThreads = 32 * kSweepWarps;  // a CTA computes 32 rows of one block

__device__ __forceinline__ double2 ldcg(const double2 *p) { return __ldcg(p); }
__device__ __forceinline__ float2 ldcg(const float2 *p) { return __ldcg(p); }
__device__ __forceinline__ void stcg(double2 *p, double2 v) { __stcg(p, v); }
__device__ __forceinline__ void stcg(float2 *p, float2 v) { __stcg(p, v); }

// Rows [r0, r0+32) of M1 v1 (+ M2 v2): lane = row, warp w = column range; column-major
// S x S blocks so every column read is a coalesced 32-row segment.  The partial sums
// of the warps are combined through shared memory; the result is returned to the
// lanes of warp 0 (row r0 + lane).
template <typename C>
__device__ __forceinline__ C tile_gemv(const C *__restrict__ M1, const C *__restrict__ v1, const C *__restrict__ M2,
                                       const C *__restrict__ v2, int S, int r0, C (*red)[33]) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int r = r0 + lane;
    const int cw = (S + kSweepWarps - 1) / kSweepWarps;
    const int c0 = w * cw, c1 = min(S, c0 + cw);
    C a0 = czero<C>(), a1 = czero<C>();
    if (r < S) {
        int c = c0;
        for (; c + 8 <= c1; c += 8) {
            C m[8], n[8];
#pragma unroll
            for (int t = 0; t < 8; ++t) m[t] = __ldg(M1 + r + (int64_t)(c + t) * S);
            if (M2) {
#pragma unroll
                for (int t = 0; t < 8; ++t) n[t] = __ldg(M2 + r + (int64_t)(c + t) * S);
            }
#pragma unroll
            for (int t = 0; t < 8; ++t) a0 = cfma(a0, m[t], v1[c + t]);
            if (M2) {
#pragma unroll
                for (int t = 0; t < 8; ++t) a1 = cfma(a1, n[t], v2[c + t]);
            }
        }
        for (; c < c1; ++c) {
            a0 = cfma(a0, __ldg(M1 + r + (int64_t)c * S), v1[c]);
            if (M2) a1 = cfma(a1, __ldg(M2 + r + (int64_t)c * S), v2[c]);
        }
    }
    red[w][lane] = a0 + a1;
    __syncthreads();
    C out = czero<C>();
    if (w == 0) {
#pragma unroll
        for (int k = 0; k < kSweepWarps; ++k) out = out + red[k][lane];
    }
    return out;
}

struct SweepArgs {
    int K, S, nlev;
    const BcrLevel *levs;
    const void *Dinv, *G, *H, *LU;
    const int *arow, *acol, *asplit;
    const double2 *aval;
    const double2 *b;
    const double *rscale;
    const double *bnorm;
    void *f, *z, *x;
    double2 *out;
    int accumulate;
    unsigned *bar;
    int *err;
    const int *skip;     // if non-null and set: return at once (refinement converged)
    int *count;          // sweeps that ran
    int *count_total;
};

template <typename C>
__global__ void __launch_bounds__(kSweepThreads) k_sweep(SweepArgs a) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    C *v1 = reinterpret_cast<C *>(smem_raw);
    C *v2 = v1 + a.S;
    __shared__ C red[kSweepWarps][33];
    if (a.skip && *a.skip) return;   // uniform over the grid: set by an earlier kernel
    if (a.count && blockIdx.x == 0 && threadIdx.x == 0) { atomicAdd(a.count, 1); atomicAdd(a.count_total, 1); }
    GridBarrier gb;
    gb.init(a.bar, a.err);
    const int S = a.S;
    const int64_t SS = (int64_t)S * S;
    const int ntile = (S + 31) / 32;
    const C *Dinv = static_cast<const C *>(a.Dinv), *G = static_cast<const C *>(a.G);
    const C *H = static_cast<const C *>(a.H), *LU = static_cast<const C *>(a.LU);
    C *f = static_cast<C *>(a.f), *z = static_cast<C *>(a.z), *x = static_cast<C *>(a.x);
    const double bn = *a.bnorm;
    const double bscale = (bn > 0.0) ? 1.0 / bn : 1.0;
    const double oscale = (bn > 0.0) ? bn : 1.0;
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    auto rhs0 = [&](int64_t p) -> C { return from_c128<C>((a.rscale[p] * bscale) * a.b[p]); };
    auto emit = [&](int64_t p, C v) {
        stcg(x + p, v);
        const double2 d = oscale * to_c128(v);
        a.out[p] = a.accumulate ? a.out[p] + d : d;
    };

    // ---------------------------------------------------------------- reduction
    for (int l = 0; l < a.nlev; ++l) {
        const BcrLevel lv = a.levs[l];
        // phase A: z_j = Dinv_j f_j for the odd blocks
        for (int64_t it = blockIdx.x; it < (int64_t)lv.nodd * ntile; it += gridDim.x) {
            const int64_t o = it / ntile;
            const int r0 = (int)(it - o * ntile) * 32;
            const int64_t j = (2 * o + 1) * lv.stride;
            __syncthreads();
            for (int c = tid; c < S; c += blockDim.x) v1[c] = (l == 0) ? rhs0(j * S + c) : ldcg(f + j * S + c);
            __syncthreads();
            const C v = tile_gemv<C>(Dinv + j * SS, v1, nullptr, nullptr, S, r0, red);
            if (w == 0 && r0 + lane < S) stcg(z + j * S + r0 + lane, v);
        }
        gb.sync();
        // phase B: f_i -= L_i z_jl + U_i z_jr for the even blocks
        if (l == 0) {
            // level 0: couplings from the CSR, one thread per row
            const int64_t nrow = (int64_t)lv.neven * S;
            for (int64_t t = blockIdx.x * (int64_t)blockDim.x + tid; t < nrow; t += (int64_t)gridDim.x * blockDim.x) {
                const int64_t e = t / S;
                const int r = (int)(t - e * S);
                const int64_t q = 2 * e;
                const bool hasl = q >= 1, hasr = q + 1 < lv.Kl;
                const int64_t p = q * S + r;
                C acc = czero<C>();
                const double rs = a.rscale[p];
                if (hasl)
                    for (int k = a.arow[p]; k < a.asplit[2 * p]; ++k)
                        acc = cfma(acc, from_c128<C>(rs * a.aval[k]), ldcg(z + a.acol[k]));
                if (hasr)
                    for (int k = a.asplit[2 * p + 1]; k < a.arow[p + 1]; ++k)
                        acc = cfma(acc, from_c128<C>(rs * a.aval[k]), ldcg(z + a.acol[k]));
                stcg(f + p, rhs0(p) - acc);
            }
        } else {
            for (int64_t it = blockIdx.x; it < (int64_t)lv.neven * ntile; it += gridDim.x) {
                const int64_t e = it / ntile;
                const int r0 = (int)(it - e * ntile) * 32;
                const int64_t q = 2 * e, i = q * lv.stride;
                const bool hasl = q >= 1, hasr = q + 1 < lv.Kl;
                const int64_t jl = (q - 1) * lv.stride, jr = (q + 1) * lv.stride;
                __syncthreads();
                for (int c = tid; c < S; c += blockDim.x) {
                    v1[c] = hasl ? ldcg(z + jl * S + c) : czero<C>();
                    v2[c] = hasr ? ldcg(z + jr * S + c) : czero<C>();
                }
                __syncthreads();
                const C *M1 = hasl ? LU + (lv.lu_L + q) * SS : (hasr ? LU + (lv.lu_U + q) * SS : nullptr);
                const C *V1 = hasl ? v1 : v2;
                const C *M2 = (hasl && hasr) ? LU + (lv.lu_U + q) * SS : nullptr;
                C acc = czero<C>();
                if (M1) acc = tile_gemv<C>(M1, V1, M2, v2, S, r0, red);
                if (w == 0 && r0 + lane < S) {
                    const int64_t p = i * S + r0 + lane;
                    stcg(f + p, ldcg(f + p) - acc);
                }
            }
        }
        gb.sync();
    }
    // ---------------------------------------------------------------- top block
    for (int64_t it = blockIdx.x; it < ntile; it += gridDim.x) {
        const int r0 = (int)it * 32;
        __syncthreads();
        for (int c = tid; c < S; c += blockDim.x) v1[c] = (a.nlev == 0) ? rhs0(c) : ldcg(f + c);
        __syncthreads();
        const C v = tile_gemv<C>(Dinv, v1, nullptr, nullptr, S, r0, red);
        if (w == 0 && r0 + lane < S) emit(r0 + lane, v);
    }
    // ---------------------------------------------------------------- back substitution
    for (int l = a.nlev - 1; l >= 0; --l) {
        gb.sync();
        const BcrLevel lv = a.levs[l];
        for (int64_t it = blockIdx.x; it < (int64_t)lv.nodd * ntile; it += gridDim.x) {
            const int64_t o = it / ntile;
            const int r0 = (int)(it - o * ntile) * 32;
            const int64_t q = 2 * o + 1, j = q * lv.stride;
            const bool hasr = q + 1 < lv.Kl;
            const int64_t jl = j - lv.stride, jr = j + lv.stride;
            __syncthreads();
            for (int c = tid; c < S; c += blockDim.x) {
                v1[c] = ldcg(x + jl * S + c);
                v2[c] = hasr ? ldcg(x + jr * S + c) : czero<C>();
            }
            __syncthreads();
            const C acc = tile_gemv<C>(G + j * SS, v1, hasr ? H + j * SS : nullptr, v2, S, r0, red);
            if (w == 0 && r0 + lane < S) {
                const int64_t p = j * S + r0 + lane;
                emit(p, ldcg(z + p) - acc);
            }
        }
    }
}

// max |v_p| over a padded vector -> red[blockIdx.x]
__global__ void k_absmax(int64_t np, const double2 *__restrict__ v, double *__restrict__ red) {
    double mx = 0.0;
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < np; p += (int64_t)gridDim.x * blockDim.x)
        mx = fmax(mx, fmax(fabs(v[p].x), fabs(v[p].y)));
    mx = warp_max_d(mx);
    __shared__ double sm[32];
    if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = mx;
    __syncthreads();
    if (threadIdx.x < 32) {
        double t = (threadIdx.x < (blockDim.x >> 5)) ? sm[threadIdx.x] : 0.0;
        t = warp_max_d(t);
        if (threadIdx.x == 0) red[blockIdx.x] = t;
    }
}

// max of in[0..n) into *out (single CTA)
__global__ void k_reduce_max(const double *__restrict__ in, int n, double *__restrict__ out) {
    double mx = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) mx = fmax(mx, in[i]);
    mx = warp_max_d(mx);
    __shared__ double sm[32];
    if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = mx;
    __syncthreads();
    if (threadIdx.x < 32) {
        double t = (threadIdx.x < (blockDim.x >> 5)) ? sm[threadIdx.x] : 0.0;
        t = warp_max_d(t);
        if (threadIdx.x == 0) *out = t;
    }
}

// 16 lanes per row, grid-stride over the rows.  mode 0: y = B x.  mode 1: y = A x - lam B x.
// mode 2: y = b - (A x - lam B x), and per-CTA maxima of |y| and |x| into part[2 b], part[2 b + 1].
constexpr int kRowLanes = 16;
__global__ void __launch_bounds__(256) k_spmv(int64_t np, int mode, const int *__restrict__ arow,
                                              const int *__restrict__ acol, const double2 *__restrict__ aval,
                                              const int *__restrict__ brow, const int *__restrict__ bcol,
                                              const double *__restrict__ bval, int has_b, double lre, double lim,
                                              const double2 *__restrict__ x, const double2 *__restrict__ rhs,
                                              double2 *__restrict__ y, double *__restrict__ part,
                                              const int *__restrict__ skip) {
    if (skip && *skip) return;
    const int sub = threadIdx.x & (kRowLanes - 1);
    const int64_t row0 = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) / kRowLanes;
    const int64_t rstride = ((int64_t)gridDim.x * blockDim.x) / kRowLanes;
    const int64_t nrow_iter = (np + rstride - 1) / rstride;   // same trip count for every lane
    const double2 lam = mk(lre, lim);
    double rmax = 0.0, xmax = 0.0;
    for (int64_t t = 0; t < nrow_iter; ++t) {
        const int64_t p = row0 + t * rstride;
        const bool live = p < np;
        double2 sa = mk(0.0, 0.0), sb = mk(0.0, 0.0);
        if (live) {
            if (mode != 0) {
                const int e1 = arow[p + 1];
                for (int e = arow[p] + sub; e < e1; e += kRowLanes)
                    sa = cfma(sa, __ldg(aval + e), __ldg(x + __ldg(acol + e)));
            }
            if (has_b) {
                const int e1 = brow[p + 1];
                for (int e = brow[p] + sub; e < e1; e += kRowLanes) sb = sb + __ldg(bval + e) * __ldg(x + __ldg(bcol + e));
            }
        }
#pragma unroll
        for (int o = kRowLanes / 2; o > 0; o >>= 1) {
            sa.x += __shfl_down_sync(0xffffffffu, sa.x, o, kRowLanes);
            sa.y += __shfl_down_sync(0xffffffffu, sa.y, o, kRowLanes);
            sb.x += __shfl_down_sync(0xffffffffu, sb.x, o, kRowLanes);
            sb.y += __shfl_down_sync(0xffffffffu, sb.y, o, kRowLanes);
        }
        if (live && sub == 0) {
            double2 v = (mode == 0) ? sb : sa - lam * sb;
            if (mode == 2) {
                v = rhs[p] - v;
                rmax = fmax(rmax, fmax(fabs(v.x), fabs(v.y)));
                xmax = fmax(xmax, fmax(fabs(x[p].x), fabs(x[p].y)));
            }
            y[p] = v;
        }
    }
    if (mode == 2) {
        rmax = warp_max_d(rmax);
        xmax = warp_max_d(xmax);
        __shared__ double sm[2][8];
        if ((threadIdx.x & 31) == 0) { sm[0][threadIdx.x >> 5] = rmax; sm[1][threadIdx.x >> 5] = xmax; }
        __syncthreads();
        if (threadIdx.x == 0) {
            for (int w = 1; w < (int)(blockDim.x >> 5); ++w) { rmax = fmax(rmax, sm[0][w]); xmax = fmax(xmax, sm[1][w]); }
            part[2 * blockIdx.x] = rmax;
            part[2 * blockIdx.x + 1] = xmax;
        }
    }
}

__global__ void k_gather(int64_t np, const int64_t *__restrict__ s2o, const double2 *__restrict__ orig,
                         double2 *__restrict__ padded) {
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < np; p += (int64_t)gridDim.x * blockDim.x) {
        const int64_t o = s2o[p];
        padded[p] = (o >= 0) ? orig[o] : mk(0.0, 0.0);
    }
}
__global__ void k_scatter(int64_t np, const int64_t *__restrict__ s2o, const double2 *__restrict__ padded,
                          double2 *__restrict__ orig) {
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < np; p += (int64_t)gridDim.x * blockDim.x) {
        const int64_t o = s2o[p];
        if (o >= 0) orig[o] = padded[p];
    }
}

template <typename C>
int launch_sweep(kore_plan *p, const double2 *b, const double *bnorm, double2 *x, int accumulate, const int *skip) {
    SweepArgs a;
    a.K = p->K; a.S = p->S; a.nlev = p->nlev; a.levs = p->d_lev;
    a.Dinv = p->d_Dinv; a.G = p->d_Gm; a.H = p->d_Hm; a.LU = p->d_LU;
    a.arow = p->d_arow; a.acol = p->d_acol; a.asplit = p->d_asplit; a.aval = p->d_aval;
    a.b = b; a.rscale = p->d_rscale; a.bnorm = bnorm;
    a.f = p->d_flo; a.z = p->d_zlo; a.x = p->d_xlo;
    a.out = x; a.accumulate = accumulate; a.bar = p->d_bar; a.err = p->d_err;
    a.skip = skip; a.count = &p->d_ir->sweeps; a.count_total = &p->d_ir->sweeps_total;
    const size_t smem = 2 * (size_t)p->S * sizeof(C);
    auto kern = k_sweep<C>;
    const int ti = (sizeof(C) == 16) ? 1 : 0;
    if (p->sweep_occ[ti] == 0) {
        if (smem > 48 * 1024)
            KORE_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        int occ = 0;
        KORE_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, kSweepThreads, smem));
        p->sweep_occ[ti] = std::max(1, std::min(occ, 4));
    }
    const int occ = p->sweep_occ[ti];
    KORE_CUDA_TRY(cudaMemsetAsync(p->d_bar, 0, sizeof(unsigned), p->stream));
    void *args[] = {&a};
    dim3 grid(p->num_sms * occ), block(kSweepThreads);
    KORE_CUDA_TRY(cudaLaunchCooperativeKernel((const void *)kern, grid, block, args, smem, p->stream));
    KORE_LAUNCHED(1);
    return KORE_OK;
}

int sweep(kore_plan *p, const double2 *b, const double *bnorm, double2 *x, int accumulate, const int *skip) {
    if (p->prof) KORE_TRY(kore_prof_mark(p, 0, true));
    const int s = (p->prec == KORE_PREC_FP64) ? launch_sweep<double2>(p, b, bnorm, x, accumulate, skip)
                                              : launch_sweep<float2>(p, b, bnorm, x, accumulate, skip);
    if (p->prof) KORE_TRY(kore_prof_mark(p, 0, false));
    return s;
}

// ||v||_inf of a padded vector into d_red[slot] (device)
int absmax(kore_plan *p, const double2 *v, int slot) {
    const unsigned grid = std::min<unsigned>(kore_div_up(p->np, 256), 1024u);
    k_absmax<<<grid, 256, 0, p->stream>>>(p->np, v, p->d_red + 2048);
    k_reduce_max<<<1, 1024, 0, p->stream>>>(p->d_red + 2048, (int)grid, p->d_red + slot);
    KORE_LAUNCHED(2);
    KORE_CUDA_TRY(cudaGetLastError());
    return KORE_OK;
}

unsigned spmv_grid(kore_plan *p) { return kore_div_up(p->np * kRowLanes, 256); }

}  // namespace

int kore_spmv_b(kore_plan *p, const double2 *x, double2 *y) {
    if (!p->has_b) return KORE_EINVAL;
    if (p->prof) KORE_TRY(kore_prof_mark(p, 2, true));
    k_spmv<<<spmv_grid(p), 256, 0, p->stream>>>(p->np, 0, p->d_arow, p->d_acol, p->d_aval, p->d_brow, p->d_bcol,
                                                 p->d_bval, 1, 0.0, 0.0, x, nullptr, y, nullptr, nullptr);
    KORE_LAUNCHED(1);
    if (p->prof) KORE_TRY(kore_prof_mark(p, 2, false));
    KORE_CUDA_TRY(cudaGetLastError());
    return KORE_OK;
}

int kore_spmv_pencil(kore_plan *p, double lre, double lim, const double2 *x, double2 *y) {
    k_spmv<<<spmv_grid(p), 256, 0, p->stream>>>(p->np, 1, p->d_arow, p->d_acol, p->d_aval, p->d_brow, p->d_bcol,
                                                 p->d_bval, p->has_b ? 1 : 0, lre, lim, x, nullptr, y, nullptr, nullptr);
    KORE_LAUNCHED(1);
    KORE_CUDA_TRY(cudaGetLastError());
    return KORE_OK;
}

int kore_gather(kore_plan *p, const double2 *orig, double2 *padded) {
    const unsigned grid = std::min<unsigned>(kore_div_up(p->np, 256), 2048u);
    k_gather<<<grid, 256, 0, p->stream>>>(p->np, p->d_slot2orig, orig, padded);
    KORE_LAUNCHED(1);
    KORE_CUDA_TRY(cudaGetLastError());
    return KORE_OK;
}

int kore_scatter(kore_plan *p, const double2 *padded, double2 *orig) {
    const unsigned grid = std::min<unsigned>(kore_div_up(p->np, 256), 2048u);
    k_scatter<<<grid, 256, 0, p->stream>>>(p->np, p->d_slot2orig, padded, orig);
    KORE_LAUNCHED(1);
    KORE_CUDA_TRY(cudaGetLastError());
    return KORE_OK;
}

namespace {

__global__ void k_ir_begin(IrState *st) {
    st->done = 0;
    st->prev = 1e300;
    st->applies += 1;
}

// eta = ||r||_inf / (||M||_inf ||x||_inf + ||b||_inf) from the per-CTA maxima of the
// residual kernel; stop when eta <= tol or when it no longer decreases (FP64 floor).
__global__ void k_ir_check(const double *__restrict__ part, int n, const double *__restrict__ bnorm, double minf,
                           double tol, IrState *st, double *rn) {
    if (st->done) return;
    double rm = 0.0, xm = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        rm = fmax(rm, part[2 * i]);
        xm = fmax(xm, part[2 * i + 1]);
    }
    rm = warp_max_d(rm);
    xm = warp_max_d(xm);
    __shared__ double s0[32], s1[32];
    if ((threadIdx.x & 31) == 0) { s0[threadIdx.x >> 5] = rm; s1[threadIdx.x >> 5] = xm; }
    __syncthreads();
    if (threadIdx.x != 0) return;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) { rm = fmax(rm, s0[w]); xm = fmax(xm, s1[w]); }
    const double den = minf * xm + *bnorm;
    const double eta = (den > 0.0) ? rm / den : 0.0;
    if (!(eta == eta)) {
        st->nan = 1;
        st->done = 1;
        return;
    }
    if (eta <= tol || eta > 0.9 * st->prev) {
        st->done = 1;
        st->eta_max = fmax(st->eta_max, eta);
        return;
    }
    st->prev = eta;
    st->iters += 1;
    st->iters_cur += 1;
    *rn = rm;
}

__global__ void k_ir_end(IrState *st) {
    if (st->iters_cur > st->iters_max) st->iters_max = st->iters_cur;
    st->iters_cur = 0;
}

}  // namespace

// d_red layout: [0, 2048) per-CTA partials of the residual kernel, [2048, 3072) partials
// of absmax, slots 4000.. scalars.
//
// Mixed precision: the refinement loop runs without host synchronisation.  Its length
// is bounded (kIrMax corrections); each step is a residual kernel, a convergence check
// on one CTA and a correction sweep, and once the check sets `done` the remaining
// kernels of the loop return at once.
constexpr int kIrMax = 6;
int kore_apply_inverse(kore_plan *p, const double2 *b, double2 *x, double tol) {
    if (!p->factored) return KORE_ENOTFACTORED;
    double *bn = p->d_red + 4000, *rn = p->d_red + 4001;
    KORE_TRY(absmax(p, b, 4000));
    if (p->prec != KORE_PREC_MIXED) return sweep(p, b, bn, x, 0, nullptr);
    if (!(tol > 0.0)) tol = 1e-14;
    k_ir_begin<<<1, 1, 0, p->stream>>>(p->d_ir);
    KORE_LAUNCHED(1);
    KORE_TRY(sweep(p, b, bn, x, 0, nullptr));
    double2 *r = p->d_v[5];
    const unsigned grid = spmv_grid(p);
    for (int it = 0; it < kIrMax; ++it) {
        if (p->prof) KORE_TRY(kore_prof_mark(p, 2, true));
        k_spmv<<<grid, 256, 0, p->stream>>>(p->np, 2, p->d_arow, p->d_acol, p->d_aval, p->d_brow, p->d_bcol,
                                            p->d_bval, p->has_b ? 1 : 0, p->sigma_re, p->sigma_im, x, b, r,
                                            p->d_part, &p->d_ir->done);
        k_ir_check<<<1, 1024, 0, p->stream>>>(p->d_part, (int)grid, bn, p->minf, tol, p->d_ir, rn);
        KORE_LAUNCHED(2);
        if (p->prof) KORE_TRY(kore_prof_mark(p, 2, false));
        KORE_TRY(sweep(p, r, rn, x, 1, &p->d_ir->done));
    }
    k_ir_end<<<1, 1, 0, p->stream>>>(p->d_ir);
    KORE_LAUNCHED(1);
    KORE_CUDA_TRY(cudaGetLastError());
    return KORE_OK;
}

int kore_ir_reset(kore_plan *p) {
    // everything but the lifetime sweep counter
    KORE_CUDA_TRY(cudaMemsetAsync(p->d_ir, 0, offsetof(IrState, sweeps_total), p->stream));
    return KORE_OK;
}

int kore_ir_read(kore_plan *p, IrState *out) {
    KORE_CUDA_TRY(cudaMemcpyAsync(out, p->d_ir, sizeof(IrState), cudaMemcpyDeviceToHost, p->stream));
    KORE_CUDA_TRY(cudaStreamSynchronize(p->stream));
    return KORE_OK;
}

// ---------------------------------------------------------------------------------
// Allocation-free solve: kore_solve_dev_noalloc (include/kore_gpu.h).
//
// Some callers cannot allocate device memory at the moment they need a solve: code
// that runs under a fixed memory budget or a pool it does not own, code that must not
// trigger the implicit device synchronisation of cudaMalloc/cudaFree inside a
// latency-critical loop, or a host library that is handed only a stream.  For them the
// scratch of one solve (padded right-hand side and solution, the reduction vectors of
// the sweep, the FP64 residual and the per-CTA maxima of the refinement loop, the
// grid-barrier counter, the error flag and the refinement state) lives in the
// file-scope array below instead of in buffers of the plan or of a caller.  Its size
// is fixed at kNoAllocMaxNp padded unknowns (about 1.6 MB, held by every GPU that
// loads the library until the process exits); larger problems are rejected.
// The kernels are the ones of kore_solve_dev; only their scratch pointers differ.
namespace {

constexpr int64_t kNoAllocMaxNp = 16384;
constexpr int64_t kNoAllocMaxSpmvCta = (kNoAllocMaxNp * kRowLanes + 255) / 256;

struct NoAllocScratch {
    double2 bp[kNoAllocMaxNp];      // padded right-hand side (complex128)
    double2 xp[kNoAllocMaxNp];      // padded solution
    double2 r[kNoAllocMaxNp];       // FP64 residual of the refinement loop
    double2 f[kNoAllocMaxNp];       // sweep reduction vectors, room for complex128
    double2 z[kNoAllocMaxNp];
    double2 x[kNoAllocMaxNp];
    double part[2 * kNoAllocMaxSpmvCta];   // per-CTA maxima of the residual kernel
    double red[2048 + 8];                  // ||b||_inf partials [0, 2048), then scalars
    IrState ir;
    unsigned bar[16];
    int err;
};

static __device__ __align__(256) NoAllocScratch g_noalloc_scratch;

// Device address of g_noalloc_scratch, looked up once per device (the symbol's name
// in host code is only a stand-in and must never be passed to a kernel).
std::mutex g_noalloc_mu;
NoAllocScratch *g_noalloc_addr[64] = {};

int noalloc_scratch(int device, NoAllocScratch **out) {
    if (device < 0 || device >= 64) return KORE_EINVAL;
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if (!g_noalloc_addr[device]) {
        void *ptr = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
        if (e != cudaSuccess || !ptr) {
            std::fprintf(stderr, "kore: cudaGetSymbolAddress of the no-allocation scratch failed: %s\n",
                         cudaGetErrorString(e));
            return KORE_ECUDA;
        }
        g_noalloc_addr[device] = static_cast<NoAllocScratch *>(ptr);
    }
    *out = g_noalloc_addr[device];
    return KORE_OK;
}

template <typename C>
int noalloc_sweep(kore_plan *p, NoAllocScratch *s, const double2 *b, const double *bnorm, double2 *x, int accumulate,
                  const int *skip, cudaStream_t st) {
    SweepArgs a;
    a.K = p->K; a.S = p->S; a.nlev = p->nlev; a.levs = p->d_lev;
    a.Dinv = p->d_Dinv; a.G = p->d_Gm; a.H = p->d_Hm; a.LU = p->d_LU;
    a.arow = p->d_arow; a.acol = p->d_acol; a.asplit = p->d_asplit; a.aval = p->d_aval;
    a.b = b; a.rscale = p->d_rscale; a.bnorm = bnorm;
    a.f = s->f; a.z = s->z; a.x = s->x;
    a.out = x; a.accumulate = accumulate; a.bar = s->bar; a.err = &s->err;
    a.skip = skip; a.count = &s->ir.sweeps; a.count_total = &s->ir.sweeps_total;
    const size_t smem = 2 * (size_t)p->S * sizeof(C);
    auto kern = k_sweep<C>;
    if (smem > 48 * 1024)
        KORE_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int occ = 0;
    KORE_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, kSweepThreads, smem));
    occ = std::max(1, std::min(occ, 4));
    KORE_CUDA_TRY(cudaMemsetAsync(s->bar, 0, sizeof(unsigned), st));
    void *args[] = {&a};
    dim3 grid(p->num_sms * occ), block(kSweepThreads);
    KORE_CUDA_TRY(cudaLaunchCooperativeKernel((const void *)kern, grid, block, args, smem, st));
    KORE_LAUNCHED(1);
    return KORE_OK;
}

int noalloc_solve(kore_plan *p, NoAllocScratch *s, const double2 *b_dev, double2 *x_dev, double tol, cudaStream_t st) {
    const bool mixed = p->prec == KORE_PREC_MIXED;
    const unsigned g = std::min<unsigned>(kore_div_up(p->np, 256), 1024u);
    double *bn = s->red + 2048, *rn = s->red + 2049;
    // every call starts from a cleared error flag and refinement state
    KORE_CUDA_TRY(cudaMemsetAsync(&s->err, 0, sizeof(int), st));
    KORE_CUDA_TRY(cudaMemsetAsync(&s->ir, 0, sizeof(IrState), st));
    k_gather<<<std::min<unsigned>(kore_div_up(p->np, 256), 2048u), 256, 0, st>>>(p->np, p->d_slot2orig, b_dev, s->bp);
    k_absmax<<<g, 256, 0, st>>>(p->np, s->bp, s->red);
    k_reduce_max<<<1, 1024, 0, st>>>(s->red, (int)g, bn);
    KORE_LAUNCHED(3);
    if (!mixed) {
        KORE_TRY(noalloc_sweep<double2>(p, s, s->bp, bn, s->xp, 0, nullptr, st));
    } else {
        if (!(tol > 0.0)) tol = 1e-14;
        k_ir_begin<<<1, 1, 0, st>>>(&s->ir);
        KORE_LAUNCHED(1);
        KORE_TRY(noalloc_sweep<float2>(p, s, s->bp, bn, s->xp, 0, nullptr, st));
        const unsigned grid = kore_div_up(p->np * kRowLanes, 256);
        for (int it = 0; it < kIrMax; ++it) {
            k_spmv<<<grid, 256, 0, st>>>(p->np, 2, p->d_arow, p->d_acol, p->d_aval, p->d_brow, p->d_bcol, p->d_bval,
                                         p->has_b ? 1 : 0, p->sigma_re, p->sigma_im, s->xp, s->bp, s->r, s->part,
                                         &s->ir.done);
            k_ir_check<<<1, 1024, 0, st>>>(s->part, (int)grid, bn, p->minf, tol, &s->ir, rn);
            KORE_LAUNCHED(2);
            KORE_TRY(noalloc_sweep<float2>(p, s, s->r, rn, s->xp, 1, &s->ir.done, st));
        }
    }
    k_scatter<<<std::min<unsigned>(kore_div_up(p->np, 256), 2048u), 256, 0, st>>>(p->np, p->d_slot2orig, s->xp, x_dev);
    KORE_LAUNCHED(1);
    KORE_CUDA_TRY(cudaGetLastError());
    return KORE_OK;
}

}  // namespace

extern "C" int kore_solve_dev_noalloc(kore_plan *p, const void *b_dev, void *x_dev, double refine_tol, void *stream) {
    if (!p || !b_dev || !x_dev) return KORE_EINVAL;
    if (p->np > kNoAllocMaxNp) {
        std::fprintf(stderr,
                     "kore_solve_dev_noalloc: %lld padded unknowns exceed the fixed scratch of %lld; "
                     "use kore_solve_dev\n",
                     (long long)p->np, (long long)kNoAllocMaxNp);
        return KORE_EINVAL;
    }
    if (!p->factored) return KORE_ENOTFACTORED;
    int prev = -1;
    cudaGetDevice(&prev);
    if (prev != p->device) KORE_CUDA_TRY(cudaSetDevice(p->device));
    NoAllocScratch *s = nullptr;
    int rc = noalloc_scratch(p->device, &s);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (rc == KORE_OK) rc = noalloc_solve(p, s, static_cast<const double2 *>(b_dev), static_cast<double2 *>(x_dev),
                                          refine_tol, st);
    if (rc == KORE_OK) {
        // wait for this call's kernels, then read its error flag and NaN state
        int flags[2] = {0, 0};
        if (cudaMemcpyAsync(&flags[0], &s->err, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
            cudaMemcpyAsync(&flags[1], &s->ir.nan, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
            cudaStreamSynchronize(st) != cudaSuccess)
            rc = KORE_ECUDA;
        else if (flags[0] != 0)
            rc = KORE_ETIMEOUT;
        else if (flags[1] != 0)
            rc = KORE_ENAN;
    }
    if (prev >= 0 && prev != p->device) cudaSetDevice(prev);
    return rc;
}
