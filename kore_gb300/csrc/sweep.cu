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

namespace {

constexpr int kSweepThreads = 128;   // one row of a block per thread, 128-row tiles

__device__ __forceinline__ double2 ldcg(const double2 *p) { return __ldcg(p); }
__device__ __forceinline__ float2 ldcg(const float2 *p) { return __ldcg(p); }
__device__ __forceinline__ void stcg(double2 *p, double2 v) { __stcg(p, v); }
__device__ __forceinline__ void stcg(float2 *p, float2 v) { __stcg(p, v); }

// acc += sum_c M[r + c*S] v[c] over c < S (column-major block, vector in shared memory)
template <typename C>
__device__ __forceinline__ C colmajor_dot(const C *__restrict__ M, int r, int S, const C *__restrict__ v) {
    C a0 = czero<C>(), a1 = czero<C>();
    int c = 0;
    for (; c + 8 <= S; c += 8) {
        C m[8];
#pragma unroll
        for (int t = 0; t < 8; ++t) m[t] = __ldg(M + r + (int64_t)(c + t) * S);
#pragma unroll
        for (int t = 0; t < 8; t += 2) {
            a0 = cfma(a0, m[t], v[c + t]);
            a1 = cfma(a1, m[t + 1], v[c + t + 1]);
        }
    }
    for (; c < S; ++c) a0 = cfma(a0, __ldg(M + r + (int64_t)c * S), v[c]);
    return a0 + a1;
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
};

template <typename C>
__global__ void __launch_bounds__(kSweepThreads) k_sweep(SweepArgs a) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    C *v1 = reinterpret_cast<C *>(smem_raw);
    C *v2 = v1 + a.S;
    GridBarrier gb;
    gb.init(a.bar, a.err);
    const int S = a.S;
    const int64_t SS = (int64_t)S * S;
    const int ntile = (S + kSweepThreads - 1) / kSweepThreads;
    const C *Dinv = static_cast<const C *>(a.Dinv), *G = static_cast<const C *>(a.G);
    const C *H = static_cast<const C *>(a.H), *LU = static_cast<const C *>(a.LU);
    C *f = static_cast<C *>(a.f), *z = static_cast<C *>(a.z), *x = static_cast<C *>(a.x);
    const double bn = *a.bnorm;
    const double bscale = (bn > 0.0) ? 1.0 / bn : 1.0;
    const double oscale = (bn > 0.0) ? bn : 1.0;
    const int tid = threadIdx.x;
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
            const int tile = (int)(it - o * ntile);
            const int64_t j = (2 * o + 1) * lv.stride;
            __syncthreads();
            for (int c = tid; c < S; c += blockDim.x) v1[c] = (l == 0) ? rhs0(j * S + c) : ldcg(f + j * S + c);
            __syncthreads();
            const int r = tile * kSweepThreads + tid;
            if (r < S) stcg(z + j * S + r, colmajor_dot(Dinv + j * SS, r, S, v1));
        }
        gb.sync();
        // phase B: f_i -= L_i z_jl + U_i z_jr for the even blocks
        for (int64_t it = blockIdx.x; it < (int64_t)lv.neven * ntile; it += gridDim.x) {
            const int64_t e = it / ntile;
            const int tile = (int)(it - e * ntile);
            const int64_t q = 2 * e, i = q * lv.stride;
            const bool hasl = q >= 1, hasr = q + 1 < lv.Kl;
            const int64_t jl = (q - 1) * lv.stride, jr = (q + 1) * lv.stride;
            const int r = tile * kSweepThreads + tid;
            if (l == 0) {
                if (r < S) {
                    const int64_t p = i * S + r;
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
                __syncthreads();
                for (int c = tid; c < S; c += blockDim.x) {
                    v1[c] = hasl ? ldcg(z + jl * S + c) : czero<C>();
                    v2[c] = hasr ? ldcg(z + jr * S + c) : czero<C>();
                }
                __syncthreads();
                if (r < S) {
                    C acc = czero<C>();
                    if (hasl) acc = colmajor_dot(LU + (lv.lu_L + q) * SS, r, S, v1);
                    if (hasr) acc = acc + colmajor_dot(LU + (lv.lu_U + q) * SS, r, S, v2);
                    stcg(f + i * S + r, ldcg(f + i * S + r) - acc);
                }
            }
        }
        gb.sync();
    }
    // ---------------------------------------------------------------- top block
    for (int64_t it = blockIdx.x; it < ntile; it += gridDim.x) {
        __syncthreads();
        for (int c = tid; c < S; c += blockDim.x) v1[c] = (a.nlev == 0) ? rhs0(c) : ldcg(f + c);
        __syncthreads();
        const int r = (int)it * kSweepThreads + tid;
        if (r < S) emit(r, colmajor_dot(Dinv, r, S, v1));
    }
    // ---------------------------------------------------------------- back substitution
    for (int l = a.nlev - 1; l >= 0; --l) {
        gb.sync();
        const BcrLevel lv = a.levs[l];
        for (int64_t it = blockIdx.x; it < (int64_t)lv.nodd * ntile; it += gridDim.x) {
            const int64_t o = it / ntile;
            const int tile = (int)(it - o * ntile);
            const int64_t q = 2 * o + 1, j = q * lv.stride;
            const bool hasr = q + 1 < lv.Kl;
            const int64_t jl = j - lv.stride, jr = j + lv.stride;
            __syncthreads();
            for (int c = tid; c < S; c += blockDim.x) {
                v1[c] = ldcg(x + jl * S + c);
                v2[c] = hasr ? ldcg(x + jr * S + c) : czero<C>();
            }
            __syncthreads();
            const int r = tile * kSweepThreads + tid;
            if (r < S) {
                C acc = colmajor_dot(G + j * SS, r, S, v1);
                if (hasr) acc = acc + colmajor_dot(H + j * SS, r, S, v2);
                emit(j * S + r, ldcg(z + j * S + r) - acc);
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

// 8 lanes per row.  mode 0: y = B x.  mode 1: y = A x - lam B x.
// mode 2: y = b - (A x - lam B x) and per-CTA maxima of |y| and |x| into red.
constexpr int kRowLanes = 8;
__global__ void k_spmv(int64_t np, int mode, const int *__restrict__ arow, const int *__restrict__ acol,
                       const double2 *__restrict__ aval, const int *__restrict__ brow,
                       const int *__restrict__ bcol, const double *__restrict__ bval, int has_b, double lre,
                       double lim, const double2 *__restrict__ x, const double2 *__restrict__ rhs,
                       double2 *__restrict__ y, double *__restrict__ red) {
    const int sub = threadIdx.x & (kRowLanes - 1);
    const int64_t row0 = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) / kRowLanes;
    const int64_t rstride = ((int64_t)gridDim.x * blockDim.x) / kRowLanes;
    const double2 lam = mk(lre, lim);
    double rmax = 0.0, xmax = 0.0;
    for (int64_t p = row0; p < np + ((np % rstride) ? rstride - np % rstride : 0); p += rstride) {
        const bool live = p < np;
        double2 sa = mk(0.0, 0.0), sb = mk(0.0, 0.0);
        if (live) {
            if (mode != 0)
                for (int e = arow[p] + sub; e < arow[p + 1]; e += kRowLanes) sa = cfma(sa, aval[e], x[acol[e]]);
            if (has_b)
                for (int e = brow[p] + sub; e < brow[p + 1]; e += kRowLanes) sb = sb + bval[e] * x[bcol[e]];
        }
#pragma unroll
        for (int o = kRowLanes / 2; o > 0; o >>= 1) {
            sa.x += __shfl_down_sync(0xffffffffu, sa.x, o, kRowLanes);
            sa.y += __shfl_down_sync(0xffffffffu, sa.y, o, kRowLanes);
            sb.x += __shfl_down_sync(0xffffffffu, sb.x, o, kRowLanes);
            sb.y += __shfl_down_sync(0xffffffffu, sb.y, o, kRowLanes);
        }
        if (live && sub == 0) {
            double2 v;
            if (mode == 0) v = sb;
            else v = sa - lam * sb;
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
        __shared__ double sm[2][32];
        if ((threadIdx.x & 31) == 0) { sm[0][threadIdx.x >> 5] = rmax; sm[1][threadIdx.x >> 5] = xmax; }
        __syncthreads();
        if (threadIdx.x < 32) {
            const bool in = threadIdx.x < (blockDim.x >> 5);
            double a = in ? sm[0][threadIdx.x] : 0.0, c = in ? sm[1][threadIdx.x] : 0.0;
            a = warp_max_d(a);
            c = warp_max_d(c);
            if (threadIdx.x == 0) { red[2 * blockIdx.x] = a; red[2 * blockIdx.x + 1] = c; }
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
int launch_sweep(kore_plan *p, const double2 *b, const double *bnorm, double2 *x, int accumulate) {
    SweepArgs a;
    a.K = p->K; a.S = p->S; a.nlev = p->nlev; a.levs = p->d_lev;
    a.Dinv = p->d_Dinv; a.G = p->d_Gm; a.H = p->d_Hm; a.LU = p->d_LU;
    a.arow = p->d_arow; a.acol = p->d_acol; a.asplit = p->d_asplit; a.aval = p->d_aval;
    a.b = b; a.rscale = p->d_rscale; a.bnorm = bnorm;
    a.f = p->d_flo; a.z = p->d_zlo; a.x = p->d_xlo;
    a.out = x; a.accumulate = accumulate; a.bar = p->d_bar; a.err = p->d_err;
    const size_t smem = 2 * (size_t)p->S * sizeof(C);
    auto kern = k_sweep<C>;
    const int ti = (sizeof(C) == 16) ? 1 : 0;
    if (p->sweep_occ[ti] == 0) {
        if (smem > 48 * 1024)
            KORE_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        int occ = 0;
        KORE_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, kSweepThreads, smem));
        p->sweep_occ[ti] = std::max(1, std::min(occ, 8));
    }
    const int occ = p->sweep_occ[ti];
    KORE_CUDA_TRY(cudaMemsetAsync(p->d_bar, 0, sizeof(unsigned), p->stream));
    void *args[] = {&a};
    dim3 grid(p->num_sms * occ), block(kSweepThreads);
    KORE_CUDA_TRY(cudaLaunchCooperativeKernel((const void *)kern, grid, block, args, smem, p->stream));
    KORE_LAUNCHED(1);
    return KORE_OK;
}

int sweep(kore_plan *p, const double2 *b, const double *bnorm, double2 *x, int accumulate) {
    if (p->prof) KORE_TRY(kore_prof_mark(p, 0, true));
    const int s = (p->prec == KORE_PREC_FP64) ? launch_sweep<double2>(p, b, bnorm, x, accumulate)
                                              : launch_sweep<float2>(p, b, bnorm, x, accumulate);
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

unsigned spmv_grid(kore_plan *p) {
    return std::min<unsigned>(kore_div_up(p->np * kRowLanes, 256), 1024u);
}

}  // namespace

int kore_spmv_b(kore_plan *p, const double2 *x, double2 *y) {
    if (!p->has_b) return KORE_EINVAL;
    k_spmv<<<spmv_grid(p), 256, 0, p->stream>>>(p->np, 0, p->d_arow, p->d_acol, p->d_aval, p->d_brow, p->d_bcol,
                                                 p->d_bval, 1, 0.0, 0.0, x, nullptr, y, nullptr);
    KORE_LAUNCHED(1);
    KORE_CUDA_TRY(cudaGetLastError());
    return KORE_OK;
}

int kore_spmv_pencil(kore_plan *p, double lre, double lim, const double2 *x, double2 *y) {
    k_spmv<<<spmv_grid(p), 256, 0, p->stream>>>(p->np, 1, p->d_arow, p->d_acol, p->d_aval, p->d_brow, p->d_bcol,
                                                 p->d_bval, p->has_b ? 1 : 0, lre, lim, x, nullptr, y, nullptr);
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

// d_red layout: [0, 2048) per-CTA partials of the residual kernel, [2048, 3072) partials
// of absmax, slots 4000.. scalars.
int kore_apply_inverse(kore_plan *p, const double2 *b, double2 *x, double tol, int *iters, double *resid) {
    if (!p->factored) return KORE_ENOTFACTORED;
    double *bn = p->d_red + 4000, *rn = p->d_red + 4001;
    KORE_TRY(absmax(p, b, 4000));
    KORE_TRY(sweep(p, b, bn, x, 0));
    int it = 0;
    double eta = -1.0;
    if (p->prec == KORE_PREC_MIXED) {
        if (!(tol > 0.0)) tol = 1e-14;
        double2 *r = p->d_v[5];
        const unsigned grid = spmv_grid(p);
        double prev = 1e300;
        for (it = 1; it <= 12; ++it) {
            k_spmv<<<grid, 256, 0, p->stream>>>(p->np, 2, p->d_arow, p->d_acol, p->d_aval, p->d_brow, p->d_bcol,
                                                p->d_bval, p->has_b ? 1 : 0, p->sigma_re, p->sigma_im, x, b, r,
                                                p->d_red);
            KORE_LAUNCHED(1);
            KORE_CUDA_TRY(cudaMemcpyAsync(p->h_red, p->d_red, 2 * grid * sizeof(double), cudaMemcpyDeviceToHost,
                                          p->stream));
            KORE_CUDA_TRY(cudaMemcpyAsync(p->h_red + 4000, bn, sizeof(double), cudaMemcpyDeviceToHost, p->stream));
            KORE_CUDA_TRY(cudaStreamSynchronize(p->stream));
            KORE_TRY(kore_check_device_error(p));
            double rmax = 0.0, xmax = 0.0;
            for (unsigned c = 0; c < grid; ++c) {
                rmax = std::max(rmax, p->h_red[2 * c]);
                xmax = std::max(xmax, p->h_red[2 * c + 1]);
            }
            const double bmax = p->h_red[4000];
            const double den = p->minf * xmax + bmax;
            eta = (den > 0.0) ? rmax / den : 0.0;
            if (!(eta == eta)) return KORE_ENAN;
            // converged, or no longer improving (FP64 residual floor reached)
            if (eta <= tol || eta > 0.9 * prev) break;
            prev = eta;
            KORE_CUDA_TRY(cudaMemcpyAsync(rn, &rmax, sizeof(double), cudaMemcpyHostToDevice, p->stream));
            KORE_TRY(sweep(p, r, rn, x, 1));
        }
    }
    if (iters) *iters = it;
    if (resid) *resid = eta;
    return KORE_OK;
}
